// C ABI of libmojovec_gpu.so (include/mojovec_gpu.h): contexts, the IVF-PQ,
// Flat and SQ8 indexes, k-means / PQ training and encoding primitives.
//
// Every entry point converts C++ exceptions into MV_ERR_* status codes and
// records the message for mv_last_error(). Host-pointer entry points copy
// their inputs to the device on a per-call stream, run, copy the results
// back and synchronise that stream before returning.
#include <algorithm>
#include <functional>
#include <cmath>
#include <limits>
#include <memory>
#include <new>
#include <map>
#include <unordered_map>

#include "mv_fast.h"
#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"
#include "mv_umma.h"

namespace mv {

static thread_local std::string g_last_error;
static thread_local mv_ctx* g_cur_ctx = nullptr;

void set_last_error(const std::string& msg) { g_last_error = msg; }

// cudaFuncSetAttribute applies to the current device, so the highest limit
// set so far is remembered per (device, kernel).
void raise_smem_limit(const void* kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> high;
  int dev = 0;
  MV_CHECK_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  size_t& h = high[{dev, kernel}];
  if (bytes <= h) return;
  MV_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  h = bytes;
}

long long current_wait_limit() {
  return g_cur_ctx ? g_cur_ctx->wait_limit.load(std::memory_order_relaxed) : 4000000000ll;
}

void count_launch() {
  if (g_cur_ctx) g_cur_ctx->launches.fetch_add(1, std::memory_order_relaxed);
}

struct CtxScope {
  mv_ctx* prev;
  explicit CtxScope(mv_ctx* c) : prev(g_cur_ctx) {
    g_cur_ctx = c;
    if (c) c->set_device();
  }
  ~CtxScope() { g_cur_ctx = prev; }
};

template <class F>
int32_t guard(mv_ctx* ctx, F&& f) {
  try {
    CtxScope scope(ctx);
    f();
    return MV_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return MV_ERR_OOM;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return MV_ERR_INTERNAL;
  }
}

int32_t guarded(mv_ctx* ctx, const std::function<void()>& f) { return guard(ctx, f); }

void h2d(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes) MV_CHECK_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
}
void d2h(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes) MV_CHECK_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
}
void d2d(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes) MV_CHECK_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s));
}
void sync(cudaStream_t s) { MV_CHECK_CUDA(cudaStreamSynchronize(s)); }

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11) for the k-means initialisation
// (clustering/kmeans.mojo:70-82): key = seed, counter from zero, +1 per step.
// ---------------------------------------------------------------------------
struct Philox {
  uint32_t key[2];
  uint32_t ctr[4] = {0, 0, 0, 0};
  explicit Philox(uint64_t seed) {
    key[0] = (uint32_t)seed;
    key[1] = (uint32_t)(seed >> 32);
  }
  void step(uint32_t* out) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
      if (r) {
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
      }
      uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
      uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
      uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
      uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
      c[1] = (uint32_t)p1;
      c[3] = (uint32_t)p0;
      c[0] = n0;
      c[2] = n2;
    }
    for (int i = 0; i < 4; ++i) out[i] = c[i];
    for (int i = 0; i < 4; ++i)
      if (++ctr[i] != 0) break;
  }
};
constexpr uint64_t KMEANS_SEED = 0x4D4F4A4F564543ull;

// Exact nearest-centroid assignment with launch_exact_argmin's result (mode
// 2: the coarse quantizer's k = 1 search; mode 1: the k-means rule, with the
// best distance in mind[] when mind is not null), computed through the
// certified tensor-core path of k_assign.cu where it applies: BF16 top-16
// candidates, their reference FP32 distances, and the exact SIMT argmin for
// the rows the error bound leaves open.
constexpr int ASSIGN_KC = 16;
void check_kernel_errors(mv_ctx* ctx, cudaStream_t s);
void assign_nearest(const float* x, int64_t n, int d, const float* cent, int k, int metric,
                    int mode, int32_t* assign, float* mind, cudaStream_t s) {
  if (n == 0) return;
  const int kind = metric == MV_METRIC_IP ? KIND_IP_SIMD8
                                          : (mode == 1 && d <= 4 ? KIND_L2_SHORT4 : KIND_L2_SIMD8);
  mv_ctx* ctx = g_cur_ctx;
  const bool cert = ctx && kind != KIND_L2_SHORT4 && umma_kpad(d) <= UMMA_TOPK_MAX_K && k > 2 * ASSIGN_KC &&
                    n >= 4096 && n <= 0x7fffffffll;
  if (!cert) {
    launch_exact_argmin(kind, mode, x, n, d, cent, k, d, d, assign, mind, 1, 0, 0, 0, s);
    return;
  }
  const int kp = umma_kpad(d), kc = ASSIGN_KC, ncp = next_pow2(kc);
  const int64_t chunk = std::min<int64_t>(n, 1 << 19);
  const int nseg = umma_topk_nseg(chunk, k, d, kc, ctx->num_sms);
  const int osegs = nseg * umma_topk_groups(d, kc);
  // Scratch from a leased slot (grow-only, reused across calls), bound to s.
  SlotLease lease(ctx);
  lease.use(s);
  DevBuf& buf = lease.slot->ws;
  buf.ensure(ws_bytes((size_t)k * kp, 2) + ws_bytes(k, 4) + ws_bytes(2, 8) +
             ws_bytes((size_t)chunk * kp, 2) + ws_bytes((size_t)chunk * osegs * ncp, 8) +
             2 * ws_bytes(chunk, 8) + ws_bytes(1, 4) + ws_bytes((size_t)chunk * d, 4) +
             2 * ws_bytes(chunk, 4));
  Arena ar(buf);
  __nv_bfloat16* cb = ar.take<__nv_bfloat16>((size_t)k * kp);
  float* cn = ar.take<float>(k);
  float* bounds = ar.take<float>(2);
  __nv_bfloat16* xb = ar.take<__nv_bfloat16>((size_t)chunk * kp);
  uint64_t* cand = ar.take<uint64_t>((size_t)chunk * osegs * ncp);
  uint64_t* gthr = ar.take<uint64_t>(chunk);
  int64_t* flagged = ar.take<int64_t>(chunk);
  int* nflag = ar.take<int>(1);
  float* sub_x = ar.take<float>((size_t)chunk * d);
  int32_t* sub_a = ar.take<int32_t>(chunk);
  float* sub_d = ar.take<float>(chunk);
  launch_to_bf16(cent, k, d, cb, cn, s);
  launch_cert_bounds(cn, cent, k, d, bounds, s);
  int64_t fallback = 0;
  for (int64_t r0 = 0; r0 < n; r0 += chunk) {
    const int64_t nb = std::min(chunk, n - r0);
    const float* xr = x + r0 * d;
    launch_to_bf16(xr, nb, d, xb, nullptr, s);
    launch_umma_topk(xb, nb, cb, k, d, metric, nullptr, cn, kc, nseg, nullptr,
                     osegs > 1 ? gthr : nullptr, cand, ctx->d_err.as<int>(), s);
    MV_CHECK_CUDA(cudaMemsetAsync(nflag, 0, sizeof(int), s));
    launch_assign_certify(xr, nb, d, cent, k, metric, cand, osegs * ncp, kc, bounds, assign + r0,
                          mind ? mind + r0 : nullptr, flagged, nflag, s);
    int h_nflag = 0;
    d2h(&h_nflag, nflag, sizeof(int), s);
    check_kernel_errors(ctx, s);  // syncs; a bounded wait that gave up raises
    if (h_nflag > 0) {
      launch_gather_rows(xr, d, flagged, h_nflag, sub_x, 1, 0, 0, s);
      launch_exact_argmin(kind, mode, sub_x, h_nflag, d, cent, k, d, d, sub_a,
                          mind ? sub_d : nullptr, 1, 0, 0, 0, s);
      launch_scatter_assign(sub_a, mind ? sub_d : nullptr, flagged, h_nflag, assign + r0,
                            mind ? mind + r0 : nullptr, s);
    }
    fallback += h_nflag;
  }
  ctx->assign_rows += n;
  ctx->assign_fallback += fallback;
}

// Batched plain k-means over `batch` independent problems that share n, d
// and k: x[b] at x + b*n*d, centroids[b] at cent + b*k*d, assign[b] at
// assign + b*n.
void kmeans_train_device(const float* x, int64_t n, int d, int k, int niter, int batch,
                         float* cent, int32_t* assign, DevBuf& scratch, cudaStream_t s,
                         double* d_obj = nullptr) {
  if (n == 0 || k <= 0) return;
  MV_REQUIRE(n <= 0xffffffffll, MV_ERR_UNSUPPORTED, "k-means: too many rows");
  // :70-82 initial rows
  Philox gen(KMEANS_SEED);
  uint32_t words[4];
  gen.step(words);
  const int64_t sample_offset = (int64_t)(words[0] % (uint32_t)n);
  std::vector<int64_t> idx(k);
  for (int i = 0; i < k; ++i) {
    if (i != 0 && i % 4 == 0) gen.step(words);
    idx[i] = (int64_t)(words[i % 4] % (uint32_t)n);
  }
  const size_t sums = (size_t)32 * k * d * batch;
  const size_t counts = (size_t)32 * k * batch;
  const bool obj = d_obj && batch == 1;
  scratch.ensure(ws_bytes(sums, 4) + ws_bytes(counts, 4) + ws_bytes(k, 8) +
                 (obj ? 2 * ws_bytes(n, 4) + ws_bytes(256, 8) : 0));
  Arena ar(scratch);
  float* local_sums = ar.take<float>(sums);
  int32_t* local_counts = ar.take<int32_t>(counts);
  int64_t* d_idx = ar.take<int64_t>(k);
  float* mind = obj ? ar.take<float>(n) : nullptr;
  int32_t* final_assign = obj ? ar.take<int32_t>(n) : nullptr;  // keeps `assign` of the last step
  double* part = obj ? ar.take<double>(256) : nullptr;
  h2d(d_idx, idx.data(), sizeof(int64_t) * k, s);
  launch_gather_rows(x, d, d_idx, k, cent, batch, n * d, (int64_t)k * d, s);
  const int kind = d <= 4 ? KIND_L2_SHORT4 : KIND_L2_SIMD8;  // kmeans.mojo:131-139
  for (int it = 0; it < niter; ++it) {
    if (batch == 1)
      assign_nearest(x, n, d, cent, k, MV_METRIC_L2, 1, assign, mind, s);
    else
      launch_exact_argmin(kind, 1, x, n, d, cent, k, d, d, assign, mind, batch, n * d,
                          (int64_t)k * d, n, s);
    if (obj) launch_sum_fp64(mind, n, part, d_obj + it, s);
    launch_kmeans_accumulate(x, n, d, k, assign, local_sums, local_counts, batch, n * d, n,
                             (int64_t)32 * k * d, (int64_t)32 * k, s);
    launch_kmeans_update(x, n, d, k, local_sums, local_counts, sample_offset, it, cent, batch,
                         n * d, (int64_t)32 * k * d, (int64_t)32 * k, (int64_t)k * d, s);
  }
  if (obj) {  // inertia of the final centroids
    assign_nearest(x, n, d, cent, k, MV_METRIC_L2, 1, final_assign, mind, s);
    launch_sum_fp64(mind, n, part, d_obj + niter, s);
  }
  sync(s);  // the host-side idx vector and scratch must outlive the kernels
}

// Fast k-means: BF16 tensor-core candidates (4 per row) with an exact FP32
// recheck for the assignment, deterministic FP64 sums for the update. Same
// initial rows and empty-cluster rule as the plain form. d_obj (niter + 1
// doubles, may be null): the inertia at each assignment step and of the
// final centroids.
void kmeans_train_fast(const float* x, int64_t n, int d, int k, int niter, float* cent,
                       int32_t* assign, DevBuf& scratch, mv_ctx* ctx, cudaStream_t s,
                       double* d_obj) {
  if (n == 0 || k <= 0) return;
  MV_REQUIRE(n <= 0x7fffffffll, MV_ERR_UNSUPPORTED, "fast k-means: too many rows");
  MV_REQUIRE(umma_kpad(d) <= UMMA_TOPK_MAX_K, MV_ERR_UNSUPPORTED, "fast k-means supports d <= 2048");
  Philox gen(KMEANS_SEED);  // kmeans.mojo:70-82, as in the plain form
  uint32_t words[4];
  gen.step(words);
  const int64_t sample_offset = (int64_t)(words[0] % (uint32_t)n);
  std::vector<int64_t> idx(k);
  for (int i = 0; i < k; ++i) {
    if (i != 0 && i % 4 == 0) gen.step(words);
    idx[i] = (int64_t)(words[i % 4] % (uint32_t)n);
  }
  const int kp = umma_kpad(d);
  const int kc = std::min(4, k);  // BF16 candidates per row
  const int ncp = next_pow2(kc);
  const int nseg = umma_topk_nseg(n, k, d, kc, ctx->num_sms);
  const int osegs = nseg * umma_topk_groups(d, kc);
  scratch.ensure(ws_bytes((size_t)n * kp, 2) + ws_bytes((size_t)k * kp, 2) + ws_bytes(k, 4) +
                 ws_bytes((size_t)n * osegs * ncp, 8) + ws_bytes(n, 8) + ws_bytes(n, 4) +
                 ws_bytes(k, 8) + ws_bytes(256, 8) + ws_bytes(km_sort_scratch_bytes(n, k), 1) +
                 ws_bytes(n, 4));
  Arena ar(scratch);
  __nv_bfloat16* xb = ar.take<__nv_bfloat16>((size_t)n * kp);
  __nv_bfloat16* cb = ar.take<__nv_bfloat16>((size_t)k * kp);
  float* cn = ar.take<float>(k);
  uint64_t* cand = ar.take<uint64_t>((size_t)n * osegs * ncp);
  uint64_t* gthr = osegs > 1 ? ar.take<uint64_t>(n) : nullptr;
  float* mind = ar.take<float>(n);
  int64_t* d_idx = ar.take<int64_t>(k);
  double* part = ar.take<double>(256);
  void* sort_ws = ar.take<uint8_t>(km_sort_scratch_bytes(n, k));
  int32_t* final_assign = ar.take<int32_t>(n);  // keeps `assign` of the last step
  h2d(d_idx, idx.data(), sizeof(int64_t) * k, s);
  launch_gather_rows(x, d, d_idx, k, cent, 1, n * d, (int64_t)k * d, s);
  launch_to_bf16(x, n, d, xb, nullptr, s);
  auto assign_step = [&](int32_t* out, double* obj_slot) {
    launch_to_bf16(cent, k, d, cb, cn, s);
    launch_umma_topk(xb, n, cb, k, d, MV_METRIC_L2, nullptr, cn, kc, nseg, nullptr, gthr, cand,
                     ctx->d_err.as<int>(), s);
    launch_km_recheck(x, n, d, cent, k, cand, osegs * ncp, out, mind, s);
    if (obj_slot) launch_sum_fp64(mind, n, part, obj_slot, s);
  };
  for (int it = 0; it < niter; ++it) {
    assign_step(assign, d_obj ? d_obj + it : nullptr);
    launch_km_update_fp64(x, n, d, k, assign, sample_offset, it, cent, sort_ws, s);
  }
  if (d_obj) assign_step(final_assign, d_obj + niter);
  sync(s);  // the host-side idx vector and scratch must outlive the kernels
}

// PQ training: subspace extraction then M batched k-means of 256 centroids
// (quantization/pq.mojo:45-69,125-176).
void pq_train_device(const float* x, int64_t n, int d, int M, int niter, float* pq_out,
                     DevBuf& work, DevBuf& scratch, cudaStream_t s) {
  const int dsub = d / M;
  work.ensure(ws_bytes((size_t)n * d, 4) + ws_bytes((size_t)M * n, 4));
  Arena ar(work);
  float* sub = ar.take<float>((size_t)n * d);
  int32_t* assign = ar.take<int32_t>((size_t)M * n);
  launch_split_subspaces(x, n, d, M, sub, s);
  kmeans_train_device(sub, n, dsub, 256, niter, M, pq_out, assign, scratch, s);
}

}  // namespace mv

using namespace mv;

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
void mv_ctx::set_device() const { cudaSetDevice(device); }

mv::Slot* mv_ctx::acquire() {
  Slot* pick = nullptr;
  {
    std::lock_guard<std::mutex> lk(mu);
    // Prefer an idle slot whose last call has drained.
    for (size_t i = 0; i < free_slots.size(); ++i) {
      if (cudaEventQuery(free_slots[i]->done) == cudaSuccess) {
        pick = free_slots[i];
        free_slots.erase(free_slots.begin() + i);
        break;
      }
    }
    if (!pick && (free_slots.empty() || all_slots.size() < 8)) {
      auto* s = new Slot();
      MV_CHECK_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
      MV_CHECK_CUDA(cudaEventCreateWithFlags(&s->done, cudaEventDisableTiming));
      all_slots.push_back(s);
      pick = s;
    }
    if (!pick) {
      pick = free_slots.front();
      free_slots.erase(free_slots.begin());
    }
  }
  MV_CHECK_CUDA(cudaEventSynchronize(pick->done));
  return pick;
}

void mv_ctx::release(mv::Slot* s, cudaStream_t used) {
  cudaEventRecord(s->done, used);
  std::lock_guard<std::mutex> lk(mu);
  free_slots.push_back(s);
}

extern "C" {

int32_t mv_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return MV_ERR_ARG;
  size_t n = std::min(len - 1, g_last_error.size());
  std::memcpy(buf, g_last_error.data(), n);
  buf[n] = 0;
  return MV_OK;
}

const char* mv_version(void) { return "mojovec-gb300 0.1 sm_103a"; }

int32_t mv_ctx_create(int32_t device, mv_ctx** out) {
  if (!out) return MV_ERR_ARG;
  *out = nullptr;
  return guard(nullptr, [&] {
    int count = 0;
    MV_CHECK_CUDA(cudaGetDeviceCount(&count));
    MV_REQUIRE(device >= 0 && device < count, MV_ERR_ARG, "no such CUDA device");
    auto ctx = std::make_unique<mv_ctx>();
    ctx->device = device;
    MV_CHECK_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    MV_CHECK_CUDA(cudaGetDeviceProperties(&prop, device));
    MV_REQUIRE(prop.major >= 10, MV_ERR_UNSUPPORTED,
               std::string("libmojovec_gpu targets sm_103a; device is ") + prop.name);
    ctx->num_sms = prop.multiProcessorCount;
    ctx->smem_optin = prop.sharedMemPerBlockOptin;
    MV_CHECK_CUDA(cudaStreamCreateWithFlags(&ctx->main_stream, cudaStreamNonBlocking));
    ctx->d_err.ensure(sizeof(int));
    MV_CHECK_CUDA(cudaMemset(ctx->d_err.p, 0, sizeof(int)));
    *out = ctx.release();
  });
}

int32_t mv_ctx_destroy(mv_ctx* ctx) {
  if (!ctx) return MV_ERR_ARG;
  return guard(ctx, [&] {
    cudaDeviceSynchronize();
    for (auto* s : ctx->all_slots) {
      if (s->stream) cudaStreamDestroy(s->stream);
      if (s->done) cudaEventDestroy(s->done);
      delete s;
    }
    if (ctx->main_stream) cudaStreamDestroy(ctx->main_stream);
    g_cur_ctx = nullptr;
    delete ctx;
  });
}

int32_t mv_ctx_synchronize(mv_ctx* ctx) {
  if (!ctx) return MV_ERR_ARG;
  return guard(ctx, [&] { MV_CHECK_CUDA(cudaDeviceSynchronize()); });
}

int64_t mv_ctx_kernel_launches(mv_ctx* ctx) { return ctx ? ctx->launches.load() : -1; }

int32_t mv_ctx_set_wait_limit(mv_ctx* ctx, int64_t cycles) {
  if (!ctx) return MV_ERR_ARG;
  ctx->wait_limit.store(cycles < 0 ? 4000000000ll : (long long)cycles, std::memory_order_relaxed);
  return MV_OK;
}

int32_t mv_ctx_certify_stats(mv_ctx* ctx, int64_t* out4) {
  if (!ctx || !out4) return MV_ERR_ARG;
  out4[0] = ctx->assign_rows.load();
  out4[1] = ctx->assign_fallback.load();
  out4[2] = ctx->flat_queries.load();
  out4[3] = ctx->flat_fallback.load();
  return MV_OK;
}

int32_t mv_ctx_profile(mv_ctx* ctx, int32_t enable) {
  if (!ctx) return MV_ERR_ARG;
  return guard(ctx, [&] {
    std::lock_guard<std::mutex> lk(ctx->prof_mu);
    for (auto& r : ctx->prof_pending) {
      cudaEventSynchronize(r.b);
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    ctx->prof_pending.clear();
    for (int i = 0; i < MV_STAGE_COUNT; ++i) {
      ctx->stage_ms[i] = 0.0;
      ctx->stage_n[i] = 0;
    }
    ctx->profile.store(enable != 0);
  });
}

int32_t mv_ctx_stage_times(mv_ctx* ctx, double* ms, int64_t* counts, int32_t nstages) {
  if (!ctx || nstages < 0) return MV_ERR_ARG;
  return guard(ctx, [&] {
    std::lock_guard<std::mutex> lk(ctx->prof_mu);
    for (auto& r : ctx->prof_pending) {
      MV_CHECK_CUDA(cudaEventSynchronize(r.b));
      float t = 0.0f;
      MV_CHECK_CUDA(cudaEventElapsedTime(&t, r.a, r.b));
      ctx->stage_ms[r.stage] += t;
      ctx->stage_n[r.stage] += 1;
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    ctx->prof_pending.clear();
    for (int i = 0; i < nstages && i < MV_STAGE_COUNT; ++i) {
      if (ms) ms[i] = ctx->stage_ms[i];
      if (counts) counts[i] = ctx->stage_n[i];
    }
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// IVF-PQ
// ---------------------------------------------------------------------------
namespace mv {

int effective_nprobe(const mv_ivfpq* ix, const mv_search_params* p) {
  int np = (p && p->nprobe > 0) ? p->nprobe : ix->nprobe;
  return std::min(np, ix->nlist);  // index_ivf_pq.mojo:253-254
}

void check_search_args(int64_t nq, int32_t k) {
  MV_REQUIRE(nq >= 0, MV_ERR_ARG, "query count must be non-negative");
  MV_REQUIRE(k >= 1 && k <= 2048, MV_ERR_ARG, "n_results must be between 1 and 2048.");
}

// Fills distances/labels with a constant (device).
__global__ void k_fill(float* d, int64_t* l, int64_t n, float dv) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    d[i] = dv;
    l[i] = -1;
  }
}
void launch_fill(float* d, int64_t* l, int64_t n, float dv, cudaStream_t s) {
  if (n == 0) return;
  k_fill<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d, l, n, dv);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

// Plain IVF-PQ search on device buffers (index_ivf_pq.mojo:225-360).
void scatter_rows(const void* src, int64_t n, int width_bytes, const int64_t* pos, void* dst,
                  cudaStream_t s);
void ensure_coarse(mv_ivfpq* ix, cudaStream_t s);

// The coarse quantizer search with k = nprobe (index_ivf_pq.mojo:264;
// index_ivf_flat.mojo:185-194), exact: the canonical nprobe nearest lists
// of each query in ascending (distance, list) order. Through the certified
// tensor-core path when nprobe plus a margin fits the GEMM's per-row list
// (`k_topp_certify`), the exact FP32 matrix + selection for the queries the
// bound leaves open and everywhere else. Returns false when the certified
// path does not apply (the caller runs the exact one).
bool coarse_topp_certified(mv_ctx* ctx, const float* d_q, int64_t nq, int d, const float* cent,
                           const __nv_bfloat16* cent_bf16, const float* cnorm, const float* ccert,
                           int nlist, int metric, int P, int32_t* probes, cudaStream_t s) {
  const int nc = std::min(nlist, P + std::max(16, P / 2));
  if (nc > UMMA_TOPK_MAX || nc >= nlist || umma_kpad(d) > UMMA_TOPK_MAX_K || nq > 0x7fffffffll) return false;
  const int kp = umma_kpad(d), ncp = next_pow2(nc);
  const int64_t qb = std::min<int64_t>(nq, 65536);
  // Candidates: the two-pass GEMM's lists reduced to each row's nc smallest
  // keys (nc <= 32, d <= 256), else the heap epilogue's per-segment keys;
  // either way a superset of the row's nc smallest approximate keys.
  const bool twopass = nc <= 32 && kp <= 256;
  const int nseg = twopass ? coarse_topk2_nseg(qb, nlist, d, nc, ctx->num_sms)
                           : umma_topk_nseg(qb, nlist, d, nc, ctx->num_sms);
  const int osegs = twopass ? 1 : nseg * umma_topk_groups(d, nc);
  const int lcap = twopass ? coarse_topk2_cap(nc) : 0;
  if ((int64_t)osegs * ncp > 256) return false;
  // Scratch from a leased slot (grow-only, reused across calls), bound to s.
  SlotLease lease(ctx);
  lease.use(s);
  DevBuf& buf = lease.slot->ws;
  buf.ensure(ws_bytes((size_t)qb * kp, 2) + ws_bytes((size_t)qb * osegs * ncp, 8) +
             2 * ws_bytes((size_t)qb, 8) + ws_bytes(1, 4) +
             (twopass ? ws_bytes((size_t)qb * nseg * lcap, 8) + ws_bytes((size_t)qb * nseg, 4) +
                            ws_bytes((size_t)qb, 4)
                      : 0));
  Arena ar(buf);
  __nv_bfloat16* xb = ar.take<__nv_bfloat16>((size_t)qb * kp);
  uint64_t* cand = ar.take<uint64_t>((size_t)qb * osegs * ncp);
  uint64_t* gthr = ar.take<uint64_t>((size_t)qb);
  int64_t* flagged = ar.take<int64_t>((size_t)qb);
  int* nflag = ar.take<int>(1);
  uint64_t* lists = twopass ? ar.take<uint64_t>((size_t)qb * nseg * lcap) : nullptr;
  int* counts = twopass ? ar.take<int>((size_t)qb * nseg) : nullptr;
  uint32_t* lthr = twopass ? ar.take<uint32_t>((size_t)qb) : nullptr;
  int64_t fallback = 0;
  for (int64_t q0 = 0; q0 < nq; q0 += qb) {
    const int64_t nb = std::min(qb, nq - q0);
    const float* xr = d_q + q0 * d;
    launch_to_bf16(xr, nb, d, xb, nullptr, s);
    if (twopass) {
      launch_coarse_topk2(xb, nb, cent_bf16, nlist, d, metric, cnorm, nc, nseg, lists, counts, lthr,
                          ctx->d_err.as<int>(), s);
      launch_lists_smallest(lists, counts, nseg, lcap, nb, nc, cand, s);
    } else {
      launch_umma_topk(xb, nb, cent_bf16, nlist, d, metric, nullptr, cnorm, nc, nseg, nullptr,
                       osegs > 1 ? gthr : nullptr, cand, ctx->d_err.as<int>(), s);
    }
    MV_CHECK_CUDA(cudaMemsetAsync(nflag, 0, sizeof(int), s));
    launch_topp_certify(xr, nb, d, cent, nlist, metric, cand, osegs * ncp, nc, P, ccert,
                        probes + q0 * P, flagged, nflag, s);
    int h_nflag = 0;
    d2h(&h_nflag, nflag, sizeof(int), s);
    check_kernel_errors(ctx, s);  // syncs
    if (h_nflag > 0) {  // the exact selection for the open queries
      DevBuf tmp;
      tmp.ensure(ws_bytes((size_t)h_nflag * d, 4) + ws_bytes((size_t)h_nflag * nlist, 4) +
                 ws_bytes((size_t)h_nflag * P, 8) + ws_bytes((size_t)h_nflag * P, 4));
      Arena ta(tmp);
      float* sx = ta.take<float>((size_t)h_nflag * d);
      float* dm = ta.take<float>((size_t)h_nflag * nlist);
      uint64_t* keys = ta.take<uint64_t>((size_t)h_nflag * P);
      int32_t* sp = ta.take<int32_t>((size_t)h_nflag * P);
      launch_gather_rows(xr, d, flagged, h_nflag, sx, 1, 0, 0, s);
      launch_exact_matrix(metric == MV_METRIC_L2 ? KIND_L2_SIMD8 : KIND_IP_SIMD8, sx, h_nflag, d,
                          cent, nlist, d, d, dm, nlist, s);
      launch_select_rows(dm, h_nflag, nlist, nlist, 0, P, nullptr, keys, nullptr, s);
      launch_keys_to_ids(keys, (int64_t)h_nflag * P, sp, s);
      scatter_rows(sp, h_nflag, 4 * P, flagged, probes + q0 * P, s);
      sync(s);
    }
    fallback += h_nflag;
  }
  ctx->assign_rows += nq;
  ctx->assign_fallback += fallback;
  return true;
}

void ivfpq_search_plain(mv_ivfpq* ix, const float* d_x, int64_t nq, int k, int nprobe,
                        const uint8_t* d_filter, int64_t filter_len, float* d_out,
                        int64_t* d_lab, DevBuf& ws, cudaStream_t s) {
  if (nq == 0) return;
  if (!ix->trained || ix->ntotal == 0) {  // :247-251
    launch_fill(d_out, d_lab, nq * k, 1e38f, s);
    return;
  }
  MV_REQUIRE(nprobe <= 8192, MV_ERR_UNSUPPORTED, "nprobe above 8192 is not supported on the GPU");
  const bool cert_coarse = umma_kpad(ix->d) <= UMMA_TOPK_MAX_K &&
                           std::min(ix->nlist, nprobe + std::max(16, nprobe / 2)) < ix->nlist &&
                           nprobe + std::max(16, nprobe / 2) <= UMMA_TOPK_MAX;
  if (cert_coarse) ensure_coarse(ix, s);
  // Query batches bound the coarse distance matrix to ~1.5 GB.
  int64_t qb = std::max<int64_t>(64, (int64_t)(1536ll * 1024 * 1024 / ((int64_t)ix->nlist * 4)));
  qb = std::min<int64_t>({qb, nq, 65535ll * 64});
  ws.ensure(ws_bytes((size_t)qb * ix->nlist, 4) + ws_bytes((size_t)qb * nprobe, 8) +
            ws_bytes((size_t)qb * nprobe, 4));
  Arena ar(ws);
  float* dmat = ar.take<float>((size_t)qb * ix->nlist);
  uint64_t* ckeys = ar.take<uint64_t>((size_t)qb * nprobe);
  int32_t* probes = ar.take<int32_t>((size_t)qb * nprobe);
  const int kind = ix->metric == MV_METRIC_L2 ? KIND_L2_SIMD8 : KIND_IP_SIMD8;
  for (int64_t q0 = 0; q0 < nq; q0 += qb) {
    const int64_t nb = std::min(qb, nq - q0);
    const float* xq = d_x + q0 * ix->d;
    // :264 coarse quantizer search with k = nprobe
    bool certified = false;
    if (cert_coarse) {
      StageTimer t(ix->ctx, MV_STAGE_COARSE, s);
      certified = coarse_topp_certified(ix->ctx, xq, nb, ix->d, ix->centroids.as<float>(),
                                        ix->d_cent_bf16.as<__nv_bfloat16>(), ix->d_cnorm.as<float>(),
                                        ix->d_ccert.as<float>(), ix->nlist, ix->metric, nprobe,
                                        probes, s);
    }
    if (!certified) {
      {
        StageTimer t(ix->ctx, MV_STAGE_COARSE, s);
        launch_exact_matrix(kind, xq, nb, ix->d, ix->centroids.as<float>(), ix->nlist, ix->d,
                            ix->d, dmat, ix->nlist, s);
      }
      StageTimer t(ix->ctx, MV_STAGE_SELECT, s);
      launch_select_rows(dmat, nb, ix->nlist, ix->nlist, 0, nprobe, nullptr, ckeys, nullptr, s);
      launch_keys_to_ids(ckeys, nb * nprobe, probes, s);
    }
    IvfpqScanArgs a;
    a.q = xq;
    a.nq = nb;
    a.d = ix->d;
    a.M = ix->M;
    a.dsub = ix->dsub;
    a.metric = ix->metric;
    a.centroids = ix->centroids.as<float>();
    a.pq = ix->pq.as<float>();
    a.list_off = ix->d_off.as<int64_t>();
    a.ids = ix->d_ids.as<uint32_t>();
    a.codes = ix->d_codes.as<uint8_t>();
    a.probes = probes;
    a.nprobe = nprobe;
    a.filter = d_filter;
    a.filter_len = d_filter ? filter_len : 0;
    a.k = k;
    a.out_d = d_out + q0 * k;
    a.out_l = d_lab + q0 * k;
    StageTimer t(ix->ctx, MV_STAGE_SCAN, s);
    launch_ivfpq_scan_plain(a, s);
  }
}

// Reads and clears the context's kernel error flag (after a stream sync).
void check_kernel_errors(mv_ctx* ctx, cudaStream_t s) {
  int e = 0;
  d2h(&e, ctx->d_err.p, sizeof(int), s);
  sync(s);
  if (e) {
    MV_CHECK_CUDA(cudaMemsetAsync(ctx->d_err.p, 0, sizeof(int), s));
    sync(s);
    if (e == 1)
      throw Error(MV_ERR_TIMEOUT, "a tensor-core kernel gave up waiting (bounded wait expired)");
    throw Error(MV_ERR_INTERNAL, "a kernel skipped an out-of-range index (site " + std::to_string(e) + ")");
  }
}

// Builds the fast-form side structures once per index state: BF16
// centroids and their norms, and the per-vector term ||y||^2 + 2<c, y>.
// Centroid-only tensor-core state: BF16 centroids, their norms and the
// certificate bounds (caller holds fast_mu).
void build_coarse_locked(mv_ivfpq* ix, cudaStream_t s) {
  if (ix->coarse_ready) return;
  const int kp = umma_kpad(ix->d);
  ix->d_cent_bf16.ensure((size_t)ix->nlist * kp * 2);
  ix->d_cnorm.ensure((size_t)ix->nlist * 4);
  ix->d_ccert.ensure(2 * sizeof(float));
  launch_to_bf16(ix->centroids.as<float>(), ix->nlist, ix->d, ix->d_cent_bf16.as<__nv_bfloat16>(),
                 ix->d_cnorm.as<float>(), s);
  launch_cert_bounds(ix->d_cnorm.as<float>(), ix->centroids.as<float>(), ix->nlist, ix->d,
                     ix->d_ccert.as<float>(), s);
  sync(s);
  ix->coarse_ready = true;
}

void ensure_coarse(mv_ivfpq* ix, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(ix->fast_mu);
  build_coarse_locked(ix, s);
}

void ensure_fast(mv_ivfpq* ix, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(ix->fast_mu);
  if (ix->fast_ready) return;
  build_coarse_locked(ix, s);
  const int64_t total = ix->h_off[ix->nlist];
  {
    std::vector<int64_t> len(ix->nlist);
    for (int L = 0; L < ix->nlist; ++L) len[L] = ix->h_off[L + 1] - ix->h_off[L];
    std::sort(len.begin(), len.end(), std::greater<int64_t>());
    ix->longest.assign(ix->nlist + 1, 0);
    for (int L = 0; L < ix->nlist; ++L) ix->longest[L + 1] = ix->longest[L] + len[L];
  }
  if (ix->metric == MV_METRIC_L2 && total > 0) {
    ix->d_vec_term.ensure((size_t)total * 4 + 16);  // staged scans copy 16-byte supersets
    launch_vec_terms(ix->d_off.as<int64_t>(), ix->nlist, ix->d_codes.as<uint8_t>(),
                     ix->pq.as<float>(), ix->centroids.as<float>(), ix->d, ix->M,
                     ix->d_vec_term.as<float>(), s);
  }
  // FP16 codebook for the fast form's per-query tables, scaled by 2^e so
  // the largest magnitude lies in [2^13, 2^14): no overflow, and the scale
  // divides out exactly.
  ix->pq16_inv = 0.0f;
  ix->has_pq_cn = false;
  const int dsub = ix->d / ix->M;
  {
    // Per subspace, the largest codeword norm (in double, rounded up): the
    // bound that scales the rotated-table scan's integer tables.
    const size_t npq = (size_t)ix->M * 256 * dsub;
    std::vector<float> h(npq);
    d2h(h.data(), ix->pq.p, sizeof(float) * npq, s);
    sync(s);
    std::vector<float> cn(ix->M);
    bool ok = true;
    for (int m = 0; m < ix->M; ++m) {
      double mx = 0.0;
      for (int c = 0; c < 256; ++c) {
        double s2 = 0.0;
        for (int t = 0; t < dsub; ++t) {
          const double v = h[((size_t)m * 256 + c) * dsub + t];
          s2 += v * v;
        }
        mx = std::max(mx, s2);
      }
      const double nrm = std::sqrt(mx) * (1.0 + 1e-6);
      ok = ok && std::isfinite(nrm) && nrm < 1e37;
      cn[m] = (float)nrm;
    }
    if (ok) {
      ix->d_pq_cn.ensure((size_t)ix->M * 4);
      h2d(ix->d_pq_cn.p, cn.data(), (size_t)ix->M * 4, s);
      sync(s);
      ix->has_pq_cn = true;
    }
  }
  if (dsub == 4 || dsub == 8) {
    const size_t npq = (size_t)ix->M * 256 * dsub;
    std::vector<float> h(npq);
    d2h(h.data(), ix->pq.p, sizeof(float) * npq, s);
    sync(s);
    float amax = 0.0f;
    bool finite = true;
    for (float v : h) {
      finite = finite && std::isfinite(v);
      amax = std::max(amax, std::fabs(v));
    }
    if (finite && amax > 0.0f && amax < 1e30f && amax > 1e-30f) {
      const int e = 13 - std::ilogb(amax);
      const float scale = std::ldexp(1.0f, e);
      std::vector<__half> h16(npq);
      for (size_t i = 0; i < npq; ++i) h16[i] = __float2half_rn(h[i] * scale);
      ix->d_pq16.ensure(npq * sizeof(__half));
      h2d(ix->d_pq16.p, h16.data(), npq * sizeof(__half), s);
      sync(s);  // the host copy goes out of scope
      ix->pq16_inv = std::ldexp(1.0f, -e);
    }
  }
  if (ix->has_raw && total > 0) {
    ix->d_raw8.ensure((size_t)total * rerank8_row_bytes(ix->d));
    ix->d_rmeta.ensure((size_t)total * sizeof(float2));
    ix->d_dim8.ensure((size_t)ix->d * sizeof(float2));
    ix->d_dimord.ensure((size_t)ix->d * 8);
    launch_rerank_rows8(ix->d_raw.as<float>(), total, ix->d, ix->d_dimord.as<uint32_t>(),
                        ix->d_dim8.as<float2>(), ix->d_raw8.as<uint8_t>(),
                        ix->d_rmeta.as<float2>(), s);
  }
  sync(s);
  ix->fast_ready = true;
}

// Fast-form IVF-PQ search (BF16 coarse GEMM + exact FP32 recheck, one LUT
// per query with precomputed per-vector terms, exact FP32 rerank). With
// `batch`, queries carry their own nprobe (<= nprobe) and k (<= k; each
// result row keeps k slots), the scan runs as a persistent grid that takes
// queries in batch->order from a counter, and the launch shapes come from
// batch (the tuner's choice). The whole batch is one chunk then, and the
// call makes no allocation, host read or synchronisation once the
// workspace is sized, so it can be captured in a CUDA graph.
void ivfpq_search_fast(mv_ivfpq* ix, const float* d_x, int64_t nq, int k, int nprobe,
                       const mv_search_params* p, float* d_out, int64_t* d_lab, DevBuf& ws,
                       cudaStream_t s, const FastBatch* batch = nullptr,
                       const uint8_t* d_filter = nullptr, int64_t filter_len = 0) {
  if (nq == 0) return;
  if (!ix->trained || ix->ntotal == 0) {
    launch_fill(d_out, d_lab, nq * k, 1e38f, s);
    return;
  }
  if (!batch) ensure_fast(ix, s);
  MV_REQUIRE(ix->has_raw || !(p && p->rerank > 0), MV_ERR_STATE,
             "the exact rerank needs the index's rows, which a snapshot does not carry; "
             "search with rerank 0");
  const bool fp32_coarse = p && p->coarse_fp32;
  const int R = std::max(k, (p && p->rerank > 0) ? (int)p->rerank : k);
  MV_REQUIRE(R <= 4096, MV_ERR_ARG, "rerank depth must be at most 4096");
  MV_REQUIRE(nprobe <= 8192, MV_ERR_UNSUPPORTED, "nprobe above 8192 is not supported on the GPU");
  const int nc = fp32_coarse ? nprobe : std::min(ix->nlist, nprobe + std::max(8, nprobe / 4));
  const int kp = umma_kpad(ix->d);
  // BF16 coarse step, three kinds that keep the same approximate top-nc
  // lists per query: the two-pass GEMM with per-row lists (nc <= 32,
  // d <= 256; coarse_path 3), the GEMM with a per-row heap epilogue
  // (nc <= 64; coarse_path 1) and the distance matrix with one warp per
  // query selecting (coarse_path 2). Automatic: two-pass where it applies,
  // else the matrix.
  const int cpath = p ? p->coarse_path : 0;
  MV_REQUIRE(cpath >= 0 && cpath <= 3, MV_ERR_ARG, "coarse_path must be 0, 1, 2 or 3");
  const bool twopass_ok = !fp32_coarse && nc <= 32 && kp <= 256;
  const bool gemm = !fp32_coarse && (batch ? !batch->coarse_matrix : cpath != 2);
  const bool twopass = gemm && twopass_ok && cpath != 1;
  const bool fused = gemm && !twopass && nc <= 64 && (batch || cpath == 1);
  int64_t qb = std::max<int64_t>(128, (int64_t)(1536ll * 1024 * 1024 / ((int64_t)ix->nlist * 4)));
  qb = std::min<int64_t>({qb, nq, 65535ll * 64});
  if (batch) {
    MV_REQUIRE(nq <= 65535ll * 64, MV_ERR_UNSUPPORTED, "batch too large for one launch");
    qb = nq;
  }
  // The two-kernel scan (distance rows, then a per-query select; the same
  // shortlist as the single-kernel scan): always with lut 7, and by default
  // (lut 0) where a query has at most 16 384 candidates and the rows of a
  // chunk of queries fit 1 GB (measured at 1M x 128, nprobe 8: scan 0.329 ms
  // against 0.341 ms; at nprobe up to 256 the rows are too long to pay).
  const int lut = p ? p->lut_fp16 : 0;
  const int64_t smax = ix->longest.empty() ? 0 : ix->longest[std::min(nprobe, ix->nlist)];
  const int64_t rstride = smax > 0 ? ivfpq_rows_stride(smax) : 0;
  constexpr int64_t kRowWords = 1ll << 28;
  const bool rows = smax > 0 && (lut == 7 || (lut == 0 && smax <= 16384 &&
                                              (batch ? nq : std::min<int64_t>(qb, 1024)) * rstride <= kRowWords));
  if (rows && !batch) qb = std::max<int64_t>(1, std::min<int64_t>(qb, kRowWords / rstride));
  const int nseg = fused ? umma_topk_nseg(qb, ix->nlist, ix->d, nc, ix->ctx->num_sms)
                 : twopass ? coarse_topk2_nseg(qb, ix->nlist, ix->d, nc, ix->ctx->num_sms) : 1;
  const int ncand = nseg * (fused ? umma_topk_groups(ix->d, nc) : 1) * next_pow2(nc);
  const int lcap = twopass ? coarse_topk2_cap(nc) : 0;
  ws.ensure(ws_bytes((size_t)qb * kp, 2) +
            (fused     ? ws_bytes((size_t)qb * ncand, 8) + ws_bytes((size_t)qb, 8)
             : twopass ? ws_bytes((size_t)qb * nseg * lcap, 8) + ws_bytes((size_t)qb * nseg, 4) +
                            ws_bytes((size_t)qb, 4)
                       : ws_bytes((size_t)qb * ix->nlist, 4)) +
            ws_bytes((size_t)qb * nprobe, 4) * 2 + ws_bytes((size_t)qb * R, 8) +
            (rows ? ws_bytes((size_t)qb * rstride, 4) : 0));
  Arena ar(ws);
  __nv_bfloat16* xq = ar.take<__nv_bfloat16>((size_t)qb * kp);
  float* dmat = fused || twopass ? nullptr : ar.take<float>((size_t)qb * ix->nlist);
  uint64_t* ckeys = fused ? ar.take<uint64_t>((size_t)qb * ncand) : nullptr;
  uint64_t* gthr = fused && ncand > next_pow2(nc) ? ar.take<uint64_t>((size_t)qb) : nullptr;
  uint64_t* clists = twopass ? ar.take<uint64_t>((size_t)qb * nseg * lcap) : nullptr;
  int* ccounts = twopass ? ar.take<int>((size_t)qb * nseg) : nullptr;
  uint32_t* cthr = twopass ? ar.take<uint32_t>((size_t)qb) : nullptr;
  int32_t* probes = ar.take<int32_t>((size_t)qb * nprobe);
  float* term = ar.take<float>((size_t)qb * nprobe);
  uint64_t* skeys = ar.take<uint64_t>((size_t)qb * R);
  uint32_t* drows = rows ? ar.take<uint32_t>((size_t)qb * rstride) : nullptr;
  for (int64_t q0 = 0; q0 < nq; q0 += qb) {
    const int64_t nb = std::min(qb, nq - q0);
    const float* xb = d_x + q0 * ix->d;
    {
      StageTimer t(ix->ctx, MV_STAGE_COARSE, s);
      if (fp32_coarse) {
        launch_exact_matrix(ix->metric == MV_METRIC_L2 ? KIND_L2_SIMD8 : KIND_IP_SIMD8, xb, nb,
                            ix->d, ix->centroids.as<float>(), ix->nlist, ix->d, ix->d, dmat,
                            ix->nlist, s);
      } else {
        launch_to_bf16(xb, nb, ix->d, xq, nullptr, s);
        if (twopass)
          launch_coarse_topk2(xq, nb, ix->d_cent_bf16.as<__nv_bfloat16>(), ix->nlist, ix->d,
                              ix->metric, ix->d_cnorm.as<float>(), nc, nseg, clists, ccounts,
                              cthr, ix->ctx->d_err.as<int>(), s);
        else if (fused)
          launch_umma_topk(xq, nb, ix->d_cent_bf16.as<__nv_bfloat16>(), ix->nlist, ix->d,
                           ix->metric, nullptr, ix->d_cnorm.as<float>(), nc, nseg, nullptr, gthr,
                           ckeys, ix->ctx->d_err.as<int>(), s);
        else if (kp > 256)  // the matrix GEMM keeps K resident: exact rows past d = 256
          launch_exact_matrix(ix->metric == MV_METRIC_L2 ? KIND_L2_SIMD8 : KIND_IP_SIMD8, xb, nb,
                              ix->d, ix->centroids.as<float>(), ix->nlist, ix->d, ix->d, dmat,
                              ix->nlist, s);
        else
          launch_umma_dist(EPI_MATRIX, xq, nb, ix->d_cent_bf16.as<__nv_bfloat16>(), ix->nlist,
                           ix->d, ix->metric, nullptr, ix->d_cnorm.as<float>(), dmat, ix->nlist,
                           nullptr, ix->ctx->d_err.as<int>(), ix->ctx->num_sms, s);
      }
    }
    {
      StageTimer t(ix->ctx, MV_STAGE_SELECT, s);
      if (twopass)
        launch_coarse_lists(clists, ccounts, nseg, lcap, nb, ix->nlist, xb, ix->d,
                            ix->centroids.as<float>(), ix->metric, nc, nprobe, probes, term,
                            ix->ctx->d_err.as<int>(), s);
      else if (fused)
        launch_coarse_from_keys(ckeys, nb, ncand, xb, ix->d, ix->centroids.as<float>(), ix->nlist,
                                ix->metric, nc, nprobe, probes, term, ix->ctx->d_err.as<int>(), s);
      else if (nc <= 64)
        launch_coarse_rows(dmat, nb, ix->nlist, xb, ix->d, ix->centroids.as<float>(), ix->metric,
                           nc, nprobe, probes, term, ix->ctx->d_err.as<int>(), s);
      else
        launch_coarse_fast(dmat, nb, ix->nlist, xb, ix->d, ix->centroids.as<float>(), ix->metric,
                           nc, nprobe, probes, term, ix->ctx->d_err.as<int>(), s);
    }
    {
      StageTimer t(ix->ctx, MV_STAGE_SCAN, s);
      FastScanArgs a;
      a.q = xb;
      a.nq = nb;
      a.d = ix->d;
      a.M = ix->M;
      a.metric = ix->metric;
      a.pq = ix->pq.as<float>();
      if (ix->pq16_inv > 0.0f) {
        a.pq16 = ix->d_pq16.as<__half>();
        a.pq16_inv = ix->pq16_inv;
      }
      if (ix->has_pq_cn) a.pq_cn = ix->d_pq_cn.as<float>();
      a.list_off = ix->d_off.as<int64_t>();
      a.codes = ix->d_codes.as<uint8_t>();
      a.vterm = ix->metric == MV_METRIC_L2 ? ix->d_vec_term.as<float>() : nullptr;
      a.probes = probes;
      a.term = term;
      a.nprobe = nprobe;
      a.R = R;
      a.sorted = (p && p->rerank > 0) ? 0 : 1;
      a.out_keys = skeys;
      a.nlist = ix->nlist;
      a.ntotal = ix->h_off[ix->nlist];
      a.err = ix->ctx->d_err.as<int>();
      if (d_filter && filter_len > 0) {
        a.filter = d_filter;
        a.filter_len = filter_len;
        a.ids = ix->d_ids.as<uint32_t>();
      }
      if (rows) {
        a.nprobe_q = batch ? batch->nprobe_q : nullptr;
        // 128 threads per query (eight queries per SM) measured 0.309 ms
        // for the scan stage at 1M x 128, nprobe 8; 256: 0.326, 512: 0.381
        launch_ivfpq_scan_rows(a, drows, smax, s, batch ? batch->scan_threads : 128, ix->ctx);
      } else if (batch) {
        a.nprobe_q = batch->nprobe_q;
        a.order = batch->order;
        a.counter = batch->scan_ctas_per_sm > 0 ? batch->counter : nullptr;
        if (a.counter) MV_CHECK_CUDA(cudaMemsetAsync(a.counter, 0, sizeof(int), s));
        launch_ivfpq_scan_fast(a, s, batch->scan_threads,
                               batch->scan_ctas_per_sm * ix->ctx->num_sms, p ? p->lut_fp16 : 0);
      } else {
        launch_ivfpq_scan_fast(a, s, 256, 0, p ? p->lut_fp16 : 0);
      }
    }
    if (p && p->rerank > 0) {
      StageTimer t(ix->ctx, MV_STAGE_RERANK, s);
      RerankArgs r;
      r.q = xb;
      r.nq = nb;
      r.d = ix->d;
      r.metric = ix->metric;
      r.raw = ix->d_raw.as<float>();
      r.ids = ix->d_ids.as<uint32_t>();
      r.cand = skeys;
      r.R = R;
      r.k = k;
      r.out_d = d_out + q0 * k;
      r.out_l = d_lab + q0 * k;
      r.ntotal = ix->h_off[ix->nlist];
      r.err = ix->ctx->d_err.as<int>();
      r.k_q = batch ? batch->k_q : nullptr;
      if (!(p && p->rerank_fp32) && ix->d_raw8.p) {
        r.raw8 = ix->d_raw8.as<uint8_t>();
        r.rmeta = ix->d_rmeta.as<float2>();
        r.dim8 = ix->d_dim8.as<float2>();
        r.d8 = rerank8_row_bytes(ix->d);
      }
      launch_rerank_fast(r, s);
    } else {
      launch_short_to_results(skeys, nb, R, k, ix->d_ids.as<uint32_t>(), ix->metric,
                              d_out + q0 * k, d_lab + q0 * k, s, batch ? batch->k_q : nullptr);
    }
  }
}

void ivfpq_search_any(mv_ivfpq* ix, const float* d_x, int64_t nq, int k,
                      const uint8_t* d_filter, int64_t filter_len, const mv_search_params* p,
                      float* d_out, int64_t* d_lab, DevBuf& ws, cudaStream_t s) {
  const int form = p ? p->form : MV_FORM_PLAIN;
  const int nprobe = effective_nprobe(ix, p);
  if (form == MV_FORM_FAST) {
    ivfpq_search_fast(ix, d_x, nq, k, nprobe, p, d_out, d_lab, ws, s, nullptr, d_filter,
                      filter_len);
  } else {
    MV_REQUIRE(form == MV_FORM_PLAIN, MV_ERR_ARG, "unknown search form");
    ivfpq_search_plain(ix, d_x, nq, k, nprobe, d_filter, filter_len, d_out, d_lab, ws, s);
  }
}

// Scatter of fixed-width rows: dst[pos[i]] = src[i] (width in 4-byte words).
__global__ void k_scatter_words(const uint32_t* __restrict__ src, int64_t n, int w,
                                const int64_t* __restrict__ pos, uint32_t* __restrict__ dst) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * w) return;
  int64_t i = e / w;
  int j = (int)(e - i * w);
  dst[pos[i] * w + j] = src[e];
}
__global__ void k_scatter_bytes(const uint8_t* __restrict__ src, int64_t n, int w,
                                const int64_t* __restrict__ pos, uint8_t* __restrict__ dst) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * w) return;
  int64_t i = e / w;
  int j = (int)(e - i * w);
  dst[pos[i] * w + j] = src[e];
}
void scatter_rows(const void* src, int64_t n, int width_bytes, const int64_t* pos, void* dst,
                  cudaStream_t s) {
  int64_t total;
  if (n == 0) return;
  if (width_bytes % 4 == 0) {
    int w = width_bytes / 4;
    total = n * w;
    k_scatter_words<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(
        static_cast<const uint32_t*>(src), n, w, pos, static_cast<uint32_t*>(dst));
  } else {
    total = n * width_bytes;
    k_scatter_bytes<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(
        static_cast<const uint8_t*>(src), n, width_bytes, pos, static_cast<uint8_t*>(dst));
  }
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

// Device list-append layout (k_lists.cu): the rebuilt CSR positions of the
// old entries, then of the n new ones, and the new offsets (device and host).
struct AppendLayout {
  DevBuf off_d, pos_d;
  std::vector<int64_t> new_off;
  int64_t cap = 0;  // entries the rebuilt arrays hold (skipped rows parked at the end)
};
void append_layout(mv_ctx* ctx, const int32_t* d_assign, int64_t n, int nlist,
                   const int64_t* d_old_off, int64_t old_total, AppendLayout& L, cudaStream_t s) {
  StageTimer t(ctx, MV_STAGE_APPEND, s);
  L.off_d.ensure(sizeof(int64_t) * (nlist + 1));
  L.pos_d.ensure(sizeof(int64_t) * (old_total + n) + 16);
  DevBuf scratch;
  scratch.ensure(list_append_scratch_bytes(n, nlist));
  launch_list_append_layout(d_assign, n, nlist, d_old_off, old_total, L.off_d.as<int64_t>(),
                            L.pos_d.as<int64_t>(), scratch.p, s);
  L.new_off.resize(nlist + 1);
  d2h(L.new_off.data(), L.off_d.p, sizeof(int64_t) * (nlist + 1), s);
  sync(s);
  L.cap = old_total + n;
}

// IndexIVFPQ.add_with_ids (index_ivf_pq.mojo:150-213): assign with the
// index-metric quantizer, residual PQ codes, append to the lists in input
// order (storage/inverted_lists.mojo:162-186). Lists are kept as CSR on the
// device; an append rebuilds it on the device (layout, then one scatter per
// array).
void ivfpq_add(mv_ivfpq* ix, const float* x, const int64_t* ids, int64_t n) {
  if (!ix->trained || n == 0) return;  // :161
  std::vector<uint32_t> ids32(n);
  for (int64_t i = 0; i < n; ++i) {
    MV_REQUIRE(ids[i] >= 0 && ids[i] <= 0xfffffffell, MV_ERR_ARG,
               "ids must be in [0, 2^32 - 2] for the GPU index");
    ids32[i] = (uint32_t)ids[i];
  }
  SlotLease lease(ix->ctx);
  cudaStream_t s = lease.stream();
  const int d = ix->d, M = ix->M, nlist = ix->nlist;
  DevBuf new_codes, new_raw, assign_d;
  new_codes.ensure((size_t)n * M + 16);
  new_raw.ensure((size_t)n * d * 4 + 16);
  assign_d.ensure((size_t)n * 4 + 16);
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(n, (1ll << 28) / d));
  {
    DevBuf& ws = lease.slot->ws;
    ws.ensure(ws_bytes((size_t)chunk * d, 4));
    Arena ar(ws);
    float* res = ar.take<float>((size_t)chunk * d);
    for (int64_t r0 = 0; r0 < n; r0 += chunk) {
      const int64_t nb = std::min(chunk, n - r0);
      float* dx = new_raw.as<float>() + r0 * d;
      int32_t* assign = assign_d.as<int32_t>() + r0;
      h2d(dx, x + r0 * d, sizeof(float) * nb * d, s);
      {
        StageTimer t(ix->ctx, MV_STAGE_COARSE, s);  // :172 quantizer.search(x, 1)
        assign_nearest(dx, nb, d, ix->centroids.as<float>(), nlist, ix->metric, 2, assign, nullptr,
                       s);
      }
      StageTimer t(ix->ctx, MV_STAGE_ENCODE, s);
      launch_residuals(dx, nb, d, ix->centroids.as<float>(), nlist, assign, res, s);
      launch_pq_encode(res, nb, d, M, ix->pq.as<float>(), new_codes.as<uint8_t>() + r0 * M, s);
    }
  }
  // New CSR layout: old entries of list l keep their order, new ones follow
  // in input order (:199-211 appends one at a time).
  const int64_t old_total = ix->h_off[nlist];
  AppendLayout L;
  append_layout(ix->ctx, assign_d.as<int32_t>(), n, nlist, ix->d_off.as<int64_t>(), old_total, L, s);
  const int64_t cap = L.cap;
  const int64_t* pos = L.pos_d.as<int64_t>();
  DevBuf ids_d, codes_d, raw_d, ids_new;
  ids_d.ensure(sizeof(uint32_t) * cap + 16);
  codes_d.ensure((size_t)cap * M + 16);
  raw_d.ensure(sizeof(float) * cap * d + 16);
  ids_new.ensure(sizeof(uint32_t) * n + 16);
  h2d(ids_new.p, ids32.data(), sizeof(uint32_t) * n, s);
  StageTimer t(ix->ctx, MV_STAGE_APPEND, s);
  if (old_total) {
    scatter_rows(ix->d_ids.p, old_total, 4, pos, ids_d.p, s);
    scatter_rows(ix->d_codes.p, old_total, M, pos, codes_d.p, s);
    if (ix->has_raw)  // lists set without rows keep no rows for their old entries
      scatter_rows(ix->d_raw.p, old_total, 4 * d, pos, raw_d.p, s);
    else
      MV_CHECK_CUDA(cudaMemsetAsync(raw_d.p, 0, sizeof(float) * cap * d, s));
  }
  scatter_rows(ids_new.p, n, 4, pos + old_total, ids_d.p, s);
  scatter_rows(new_codes.p, n, M, pos + old_total, codes_d.p, s);
  scatter_rows(new_raw.p, n, 4 * d, pos + old_total, raw_d.p, s);
  sync(s);
  DevBuf& off_d = L.off_d;
  std::vector<int64_t>& new_off = L.new_off;
  std::swap(ix->d_off.p, off_d.p);
  std::swap(ix->d_off.bytes, off_d.bytes);
  std::swap(ix->d_ids.p, ids_d.p);
  std::swap(ix->d_ids.bytes, ids_d.bytes);
  std::swap(ix->d_codes.p, codes_d.p);
  std::swap(ix->d_codes.bytes, codes_d.bytes);
  std::swap(ix->d_raw.p, raw_d.p);
  std::swap(ix->d_raw.bytes, raw_d.bytes);
  ix->h_off = new_off;
  ix->ntotal += n;  // :213 counts every input row
  if (old_total == 0) ix->has_raw = true;  // every entry now has its row
  ix->fast_ready = false;
}

}  // namespace mv

extern "C" {

int32_t mv_ivfpq_create(mv_ctx* ctx, int32_t d, int32_t nlist, int32_t M, int32_t metric,
                        mv_ivfpq** out) {
  if (!ctx || !out) return MV_ERR_ARG;
  *out = nullptr;
  return guard(ctx, [&] {
    // index_ivf_pq.mojo:52-59 and core/validation.mojo:11-13
    MV_REQUIRE(d > 0 && d <= 65536, MV_ERR_ARG, "dimension must be between 1 and 65536.");
    MV_REQUIRE(nlist > 0 && nlist <= 1000000, MV_ERR_ARG, "IVF-PQ nlist must be between 1 and 1000000.");
    MV_REQUIRE(M > 0 && M <= d && d % M == 0, MV_ERR_ARG,
               "IVF-PQ M must divide dimension and be between 1 and dimension.");
    MV_REQUIRE(metric == MV_METRIC_L2 || metric == MV_METRIC_IP, MV_ERR_ARG, "unknown metric");
    auto ix = std::make_unique<mv_ivfpq>();
    ix->ctx = ctx;
    ix->d = d;
    ix->nlist = nlist;
    ix->M = M;
    ix->dsub = d / M;
    ix->metric = metric;
    ix->centroids.ensure(sizeof(float) * nlist * d);
    ix->pq.ensure(sizeof(float) * 256 * d);
    ix->h_off.assign(nlist + 1, 0);
    ix->d_off.ensure(sizeof(int64_t) * (nlist + 1));
    MV_CHECK_CUDA(cudaMemset(ix->d_off.p, 0, sizeof(int64_t) * (nlist + 1)));
    MV_CHECK_CUDA(cudaMemset(ix->centroids.p, 0, sizeof(float) * nlist * d));
    MV_CHECK_CUDA(cudaMemset(ix->pq.p, 0, sizeof(float) * 256 * d));
    *out = ix.release();
  });
}

int32_t mv_ivfpq_destroy(mv_ivfpq* ix) {
  if (!ix) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    cudaDeviceSynchronize();
    delete ix;
  });
}

int32_t mv_ivfpq_set_nprobe(mv_ivfpq* ix, int32_t nprobe) {
  if (!ix) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    MV_REQUIRE(nprobe >= 1 && nprobe <= 65536, MV_ERR_ARG, "nprobe must be between 1 and nlist.");
    ix->nprobe = nprobe;
  });
}

int32_t mv_ivfpq_info(mv_ivfpq* ix, int64_t* out7) {
  if (!ix || !out7) return MV_ERR_ARG;
  out7[0] = ix->d;
  out7[1] = ix->nlist;
  out7[2] = ix->M;
  out7[3] = ix->nprobe;
  out7[4] = ix->ntotal;
  out7[5] = ix->metric;
  out7[6] = ix->trained ? 1 : 0;
  return MV_OK;
}

int32_t mv_ivfpq_set_codebooks(mv_ivfpq* ix, const float* centroids, const float* pq) {
  if (!ix || !centroids || !pq) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(ix->mu);
    MV_CHECK_CUDA(cudaMemcpy(ix->centroids.p, centroids, sizeof(float) * ix->nlist * ix->d,
                             cudaMemcpyHostToDevice));
    MV_CHECK_CUDA(cudaMemcpy(ix->pq.p, pq, sizeof(float) * 256 * ix->d, cudaMemcpyHostToDevice));
    ix->trained = true;
    ix->fast_ready = false;
    ix->coarse_ready = false;
  });
}

int32_t mv_ivfpq_get_codebooks(mv_ivfpq* ix, float* centroids, float* pq) {
  if (!ix) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    if (centroids)
      MV_CHECK_CUDA(cudaMemcpy(centroids, ix->centroids.p, sizeof(float) * ix->nlist * ix->d,
                               cudaMemcpyDeviceToHost));
    if (pq)
      MV_CHECK_CUDA(cudaMemcpy(pq, ix->pq.p, sizeof(float) * 256 * ix->d, cudaMemcpyDeviceToHost));
  });
}

int32_t mv_ivfpq_set_lists(mv_ivfpq* ix, const int64_t* offsets, const int64_t* ids,
                           const uint8_t* codes) {
  if (!ix || !offsets) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(ix->mu);
    const int nlist = ix->nlist;
    MV_REQUIRE(offsets[0] == 0, MV_ERR_ARG, "list offsets must start at 0");
    for (int l = 0; l < nlist; ++l)
      MV_REQUIRE(offsets[l + 1] >= offsets[l], MV_ERR_ARG, "list offsets must not decrease");
    const int64_t total = offsets[nlist];
    MV_REQUIRE(total == 0 || (ids && codes), MV_ERR_ARG, "ids and codes are required");
    std::vector<uint32_t> ids32((size_t)total);
    for (int64_t i = 0; i < total; ++i) {
      MV_REQUIRE(ids[i] >= 0 && ids[i] <= 0xfffffffell, MV_ERR_ARG,
                 "ids must be in [0, 2^32 - 2] for the GPU index");
      ids32[(size_t)i] = (uint32_t)ids[i];
    }
    ix->d_off.ensure(sizeof(int64_t) * (nlist + 1));
    ix->d_ids.ensure(sizeof(uint32_t) * total + 16);
    ix->d_codes.ensure((size_t)total * ix->M + 16);
    MV_CHECK_CUDA(cudaMemcpy(ix->d_off.p, offsets, sizeof(int64_t) * (nlist + 1), cudaMemcpyHostToDevice));
    if (total) {
      MV_CHECK_CUDA(cudaMemcpy(ix->d_ids.p, ids32.data(), sizeof(uint32_t) * total, cudaMemcpyHostToDevice));
      MV_CHECK_CUDA(cudaMemcpy(ix->d_codes.p, codes, (size_t)total * ix->M, cudaMemcpyHostToDevice));
    }
    ix->h_off.assign(offsets, offsets + nlist + 1);
    ix->ntotal = total;
    ix->has_raw = false;  // no rows: plain search and the fast form without rerank
    ix->fast_ready = false;
  });
}

int32_t mv_ivfpq_train_ex(mv_ivfpq* ix, const float* x, int64_t n, int32_t niter_coarse,
                          int32_t niter_pq, const mv_search_params* params) {
  if (!ix || (!x && n > 0)) return MV_ERR_ARG;
  const int form = params ? params->form : MV_FORM_PLAIN;
  if (form != MV_FORM_PLAIN && form != MV_FORM_FAST) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(ix->mu);
    if (ix->trained) return;  // :93
    MV_REQUIRE(n > 0, MV_ERR_ARG, "training needs at least one vector");
    MV_REQUIRE(niter_coarse >= 0 && niter_pq >= 0, MV_ERR_ARG, "niter must be non-negative");
    SlotLease lease(ix->ctx);
    cudaStream_t s = lease.stream();
    const int d = ix->d;
    DevBuf dx, res, assign, work, scratch;
    dx.ensure(sizeof(float) * n * d);
    h2d(dx.p, x, sizeof(float) * n * d, s);
    // 1. coarse k-means (:98-103)
    assign.ensure(sizeof(int32_t) * n);
    if (form == MV_FORM_FAST && umma_kpad(d) <= UMMA_TOPK_MAX_K)
      kmeans_train_fast(dx.as<float>(), n, d, ix->nlist, niter_coarse, ix->centroids.as<float>(),
                        assign.as<int32_t>(), scratch, ix->ctx, s, nullptr);
    else
      kmeans_train_device(dx.as<float>(), n, d, ix->nlist, niter_coarse, 1,
                          ix->centroids.as<float>(), assign.as<int32_t>(), scratch, s);
    // 2. index-metric assignment and residuals (:113-128)
    assign_nearest(dx.as<float>(), n, d, ix->centroids.as<float>(), ix->nlist, ix->metric, 2,
                   assign.as<int32_t>(), nullptr, s);
    res.ensure(sizeof(float) * n * d);
    launch_residuals(dx.as<float>(), n, d, ix->centroids.as<float>(), ix->nlist,
                     assign.as<int32_t>(), res.as<float>(), s);
    dx.release();
    // 3. PQ on residuals (:130-132)
    pq_train_device(res.as<float>(), n, d, ix->M, niter_pq, ix->pq.as<float>(), work, scratch, s);
    sync(s);
    ix->trained = true;
    ix->fast_ready = false;
    ix->coarse_ready = false;
  });
}

int32_t mv_ivfpq_train(mv_ivfpq* ix, const float* x, int64_t n, int32_t niter_coarse,
                       int32_t niter_pq) {
  return mv_ivfpq_train_ex(ix, x, n, niter_coarse, niter_pq, nullptr);
}

int32_t mv_ivfpq_add_with_ids(mv_ivfpq* ix, const float* x, const int64_t* ids, int64_t n) {
  if (!ix || n < 0 || (n > 0 && (!x || !ids))) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(ix->mu);
    ivfpq_add(ix, x, ids, n);
  });
}

int32_t mv_ivfpq_add(mv_ivfpq* ix, const float* x, int64_t n) {
  if (!ix || n < 0 || (n > 0 && !x)) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(ix->mu);
    std::vector<int64_t> ids(n);
    for (int64_t i = 0; i < n; ++i) ids[i] = ix->ntotal + i;  // :144-148
    ivfpq_add(ix, x, ids.data(), n);
  });
}

int32_t mv_ivfpq_get_lists(mv_ivfpq* ix, int64_t* offsets, int64_t* ids, uint8_t* codes) {
  if (!ix) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(ix->mu);
    const int64_t total = ix->h_off[ix->nlist];
    if (offsets) std::memcpy(offsets, ix->h_off.data(), sizeof(int64_t) * (ix->nlist + 1));
    if (ids && total) {
      std::vector<uint32_t> tmp(total);
      MV_CHECK_CUDA(cudaMemcpy(tmp.data(), ix->d_ids.p, sizeof(uint32_t) * total, cudaMemcpyDeviceToHost));
      for (int64_t i = 0; i < total; ++i) ids[i] = tmp[i];
    }
    if (codes && total)
      MV_CHECK_CUDA(cudaMemcpy(codes, ix->d_codes.p, (size_t)total * ix->M, cudaMemcpyDeviceToHost));
  });
}

int32_t mv_ivfpq_search_device(mv_ivfpq* ix, const float* d_x, int64_t nq, int32_t k,
                               const uint8_t* d_filter, int64_t filter_len,
                               const mv_search_params* params, float* d_distances,
                               int64_t* d_labels, void* stream) {
  if (!ix || (nq > 0 && (!d_x || !d_distances || !d_labels))) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    check_search_args(nq, k);
    SlotLease lease(ix->ctx);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : lease.stream();
    lease.use(s);
    ivfpq_search_any(ix, d_x, nq, k, d_filter, filter_len, params, d_distances, d_labels,
                     lease.slot->ws, s);
    if (!stream) check_kernel_errors(ix->ctx, s);
  });
}

int32_t mv_ivfpq_search(mv_ivfpq* ix, const float* x, int64_t nq, int32_t k,
                        const uint8_t* filter, int64_t filter_len,
                        const mv_search_params* params, float* distances, int64_t* labels) {
  if (!ix || (nq > 0 && (!x || !distances || !labels))) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    check_search_args(nq, k);
    if (nq == 0) return;
    // Large batches run as two halves on two streams (each with its own
    // scratch), so that the second half's query copy and the first half's
    // result copy overlap the other half's kernels. A query's results do not
    // depend on the batch it is searched in.
    constexpr int64_t kOverlapMin = 8192;
    const int parts = nq >= kOverlapMin ? 2 : 1;
    std::unique_ptr<SlotLease> leases[2];
    for (int h = 0; h < parts; ++h) leases[h].reset(new SlotLease(ix->ctx));
    const size_t fl = filter ? (size_t)filter_len : 0;
    const int64_t per = (nq + parts - 1) / parts;
    for (int h = 0; h < parts; ++h) {
      const int64_t q0 = h * per, nh = std::min(per, nq - q0);
      cudaStream_t s = leases[h]->stream();
      DevBuf& io = leases[h]->slot->io;
      io.ensure(ws_bytes((size_t)nh * ix->d, 4) + ws_bytes((size_t)nh * k, 4) +
                ws_bytes((size_t)nh * k, 8) + ws_bytes(fl + 1, 1));
      Arena ar(io);
      float* dx = ar.take<float>((size_t)nh * ix->d);
      float* dd = ar.take<float>((size_t)nh * k);
      int64_t* dl = ar.take<int64_t>((size_t)nh * k);
      uint8_t* df = ar.take<uint8_t>(fl + 1);
      h2d(dx, x + q0 * ix->d, sizeof(float) * nh * ix->d, s);
      if (fl) h2d(df, filter, fl, s);
      ivfpq_search_any(ix, dx, nh, k, fl ? df : nullptr, (int64_t)fl, params, dd, dl,
                       leases[h]->slot->ws, s);
      d2h(distances + q0 * k, dd, sizeof(float) * nh * k, s);
      d2h(labels + q0 * k, dl, sizeof(int64_t) * nh * k, s);
    }
    for (int h = 0; h + 1 < parts; ++h) sync(leases[h]->stream());
    check_kernel_errors(ix->ctx, leases[parts - 1]->stream());
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Flat
// ---------------------------------------------------------------------------
namespace mv {

void flat_search_exact(mv_flat* ix, const float* d_x, int64_t nq, int k, const uint8_t* d_filter,
                       float* d_out, int64_t* d_lab, DevBuf& ws, cudaStream_t s) {
  if (nq == 0) return;
  const int64_t nb = ix->ntotal;
  if (nb == 0) {
    launch_fill(d_out, d_lab, nq * k, 0.0f, s);
    return;
  }
  int64_t qb = std::min<int64_t>(nq, 65535ll * 64);
  int64_t cb = (int64_t)(1024ll * 1024 * 1024 / 4) / std::max<int64_t>(qb, 1);
  cb = std::max<int64_t>(64, (cb / 64) * 64);
  cb = std::min(cb, nb);
  ws.ensure(ws_bytes((size_t)qb * cb, 4) + 2 * ws_bytes((size_t)qb * k, 8));
  Arena ar(ws);
  float* dmat = ar.take<float>((size_t)qb * cb);
  uint64_t* ka = ar.take<uint64_t>((size_t)qb * k);
  uint64_t* kb = ar.take<uint64_t>((size_t)qb * k);
  const int kind = ix->metric == MV_METRIC_L2 ? KIND_L2_SIMD8 : KIND_IP_SIMD8;
  for (int64_t q0 = 0; q0 < nq; q0 += qb) {
    const int64_t nqb = std::min(qb, nq - q0);
    uint64_t* cur = ka;
    uint64_t* nxt = kb;
    bool first = true;
    for (int64_t c0 = 0; c0 < nb; c0 += cb) {
      const int64_t nc = std::min(cb, nb - c0);
      {
        StageTimer t(ix->ctx, MV_STAGE_FLAT, s);
        launch_exact_matrix(kind, d_x + q0 * ix->d, nqb, ix->d, ix->rows.as<float>() + c0 * ix->d,
                            nc, ix->d, ix->d, dmat, nc, s);
      }
      StageTimer t(ix->ctx, MV_STAGE_SELECT, s);
      launch_select_rows(dmat, nqb, nc, nc, c0, k, first ? nullptr : cur, nxt, d_filter, s);
      std::swap(cur, nxt);
      first = false;
    }
    // index_flat.mojo:305-316; rows beyond ntotal read 0.0 / -1.
    launch_keys_to_results(cur, nqb, k, 0.0f, ix->metric == MV_METRIC_IP, d_out + q0 * k,
                           d_lab + q0 * k, s);
  }
}

// Fast-form side structures of a flat index: BF16 rows (padded to the
// GEMM's k-blocks) and the FP32 norms of the rounded rows.
void ensure_flat_fast(mv_flat* ix, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(ix->fast_mu);
  if (ix->fast_ready) return;
  const int kp = umma_kpad(ix->d);
  ix->rows_bf16.ensure((size_t)ix->ntotal * kp * 2);
  ix->norms.ensure((size_t)ix->ntotal * 4);
  ix->cert.ensure(2 * sizeof(float));
  launch_to_bf16(ix->rows.as<float>(), ix->ntotal, ix->d, ix->rows_bf16.as<__nv_bfloat16>(),
                 ix->norms.as<float>(), s);
  launch_cert_bounds(ix->norms.as<float>(), ix->rows.as<float>(), ix->ntotal, ix->d,
                     ix->cert.as<float>(), s);
  sync(s);
  ix->fast_ready = true;
}

void ensure_flat_e4m3(mv_flat* ix, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(ix->fast_mu);
  if (ix->e4m3_ready) return;
  ix->rows_e4m3.ensure((size_t)ix->ntotal * umma_kpad8(ix->d) + 16);
  ix->scales_e4m3.ensure((size_t)ix->ntotal * 4 + 16);
  ix->norms_e4m3.ensure((size_t)ix->ntotal * 4 + 16);
  launch_to_e4m3(ix->rows.as<float>(), ix->ntotal, ix->d, ix->rows_e4m3.as<uint8_t>(),
                 ix->scales_e4m3.as<float>(), ix->norms_e4m3.as<float>(), s);
  sync(s);
  ix->e4m3_ready = true;
}

// Plain Flat search (index_flat.mojo:260-325), bit-exact. Where it applies
// it runs on the tensor cores: the BF16 top-k GEMM keeps a shortlist of R
// rows per query, k_flat_certify computes their reference FP32 distances,
// writes the k smallest and proves with the BF16 error bound that no other
// row can rank ahead; queries the bound leaves open (or whose shortlist
// overflowed) are recomputed by the exact SIMT scan. Elsewhere the exact
// scan runs alone.
void flat_search_plain(mv_flat* ix, const float* d_x, int64_t nq, int k, const uint8_t* d_filter,
                       float* d_out, int64_t* d_lab, DevBuf& ws, cudaStream_t s) {
  if (nq == 0) return;
  const int64_t nb = ix->ntotal;
  if (nb < 4096 || k > 128 || umma_kpad(ix->d) > UMMA_TOPK_MAX_K || nb > 0xfffffffell ||
      flat_certify_smem(ix->d, 2 * std::max(k, 32), k) > 200 * 1024) {
    flat_search_exact(ix, d_x, nq, k, d_filter, d_out, d_lab, ws, s);
    return;
  }
  ensure_flat_fast(ix, s);
  const int R = k <= 32 ? std::min(64, std::max(32, 2 * k)) : 2 * k;
  const int kseg = std::min(R, UMMA_TOPK_MAX);
  const int ncp = next_pow2(kseg);
  const int kp = umma_kpad(ix->d);
  const int64_t qb = std::min<int64_t>(nq, 32768);
  int nseg = umma_topk_nseg(qb, nb, ix->d, kseg, ix->ctx->num_sms);
  const int groups = umma_topk_groups(ix->d, kseg);
  if (kseg < R) {  // as in the fast form: batch-independent segment counts
    const int64_t nct = (nb + 127) / 128;
    nseg = (int)std::min<int64_t>((R + 15) / 16 / groups + 1, std::max<int64_t>(1, nct));
  }
  const int osegs = nseg * groups;
  ws.ensure(ws_bytes((size_t)qb * kp, 2) + ws_bytes((size_t)qb * osegs * ncp, 8) +
            ws_bytes((size_t)qb * R, 8) + 2 * ws_bytes((size_t)qb, 4) + ws_bytes((size_t)qb, 8));
  Arena ar(ws);
  __nv_bfloat16* xq = ar.take<__nv_bfloat16>((size_t)qb * kp);
  uint64_t* cand = ar.take<uint64_t>((size_t)qb * osegs * ncp);
  uint64_t* skeys = ar.take<uint64_t>((size_t)qb * R);
  int* over = ar.take<int>((size_t)qb);
  int* flag = ar.take<int>((size_t)qb);
  uint64_t* gthr = (kseg == R && osegs > 1) ? ar.take<uint64_t>((size_t)qb) : nullptr;
  std::vector<int> h_flag;
  for (int64_t q0 = 0; q0 < nq; q0 += qb) {
    const int64_t nqb = std::min(qb, nq - q0);
    const float* xb = d_x + q0 * ix->d;
    {
      StageTimer t(ix->ctx, MV_STAGE_FLAT, s);
      launch_to_bf16(xb, nqb, ix->d, xq, nullptr, s);
      launch_umma_topk(xq, nqb, ix->rows_bf16.as<__nv_bfloat16>(), nb, ix->d, ix->metric, nullptr,
                       ix->norms.as<float>(), kseg, nseg, d_filter, gthr, cand,
                       ix->ctx->d_err.as<int>(), s);
    }
    {
      StageTimer t(ix->ctx, MV_STAGE_SELECT, s);
      launch_flat_merge(cand, nqb, osegs, ncp, kseg, R, skeys, k, nullptr, ix->metric, 0.0f,
                        nullptr, nullptr, kseg < R ? over : nullptr, s);
      launch_flat_certify(xb, nqb, ix->d, ix->metric, ix->rows.as<float>(), nb, skeys, R, k,
                          ix->cert.as<float>(), kseg < R ? over : nullptr, d_out + q0 * k,
                          d_lab + q0 * k, flag, s);
    }
    h_flag.resize((size_t)nqb);
    d2h(h_flag.data(), flag, sizeof(int) * nqb, s);
    check_kernel_errors(ix->ctx, s);  // syncs
    std::vector<int64_t> rows;
    for (int64_t i = 0; i < nqb; ++i)
      if (h_flag[(size_t)i]) rows.push_back(q0 + i);
    ix->ctx->flat_queries += nqb;
    ix->ctx->flat_fallback += (int64_t)rows.size();
    if (rows.empty()) continue;
    const int64_t nr = (int64_t)rows.size();
    DevBuf tmp, tws;
    tmp.ensure(ws_bytes((size_t)nr, 8) + ws_bytes((size_t)nr * ix->d, 4) +
               ws_bytes((size_t)nr * k, 4) + ws_bytes((size_t)nr * k, 8));
    Arena ta(tmp);
    int64_t* idx = ta.take<int64_t>((size_t)nr);
    float* tx = ta.take<float>((size_t)nr * ix->d);
    float* td = ta.take<float>((size_t)nr * k);
    int64_t* tl = ta.take<int64_t>((size_t)nr * k);
    h2d(idx, rows.data(), sizeof(int64_t) * nr, s);
    launch_gather_rows(d_x, ix->d, idx, nr, tx, 1, 0, 0, s);
    flat_search_exact(ix, tx, nr, k, d_filter, td, tl, tws, s);
    scatter_rows(td, nr, 4 * k, idx, d_out, s);
    scatter_rows(tl, nr, 8 * k, idx, d_lab, s);
    sync(s);  // tmp is freed on the next iteration
  }
}

// Flat fast form: BF16 tensor-core distances with the per-row heap epilogue
// (shortlist of R = max(k, rerank) keys per query, ranked by the BF16
// distance, ties by the smaller row), then either the exact FP32 rerank of
// the shortlist or, without rerank, the BF16 distances themselves. A query
// whose shortlist may be incomplete (a segment overflow, possible only when
// R > 64) is recomputed with the exact FP32 scan.
void flat_search_fast(mv_flat* ix, const float* d_x, int64_t nq, int k, const uint8_t* d_filter,
                      const mv_search_params* p, float* d_out, int64_t* d_lab, DevBuf& ws,
                      cudaStream_t s) {
  if (nq == 0) return;
  const int64_t nb = ix->ntotal;
  if (nb == 0) {
    launch_fill(d_out, d_lab, nq * k, 0.0f, s);
    return;
  }
  MV_REQUIRE(umma_kpad(ix->d) <= UMMA_TOPK_MAX_K, MV_ERR_UNSUPPORTED, "fast flat form supports d <= 2048");
  const bool e4m3 = p && p->flat_e4m3;
  MV_REQUIRE(!e4m3 || (p->rerank > 0), MV_ERR_UNSUPPORTED, "the E4M3 shortlist needs a rerank");
  if (e4m3) ensure_flat_e4m3(ix, s);
  else ensure_flat_fast(ix, s);
  const bool rerank = p && p->rerank > 0;
  const int R = std::max(k, rerank ? (int)p->rerank : k);
  MV_REQUIRE(R <= 4096, MV_ERR_ARG, "rerank depth must be at most 4096");
  const int kseg = std::min(R, UMMA_TOPK_MAX);
  const int ncp = next_pow2(kseg);
  const int kp = e4m3 ? umma_kpad8(ix->d) / 2 : umma_kpad(ix->d);  // BF16 elements of a query row
  const int64_t qb = std::min<int64_t>(nq, 32768);
  int nseg = umma_topk_nseg(qb, nb, ix->d, kseg, ix->ctx->num_sms, e4m3);
  const int groups = umma_topk_groups(ix->d, kseg, e4m3);
  if (kseg < R) {
    // About 16 shortlist keys per segment keeps overflow rare. The count
    // depends on the index and R only, never on the batch, so whether a
    // query overflows (and is recomputed exactly) does not depend on the
    // other queries it was batched with.
    const int64_t nct = (nb + 127) / 128;
    nseg = (int)std::min<int64_t>((R + 15) / 16 / groups + 1, std::max<int64_t>(1, nct));
  }
  const int osegs = nseg * groups;  // output segments per query
  ws.ensure(ws_bytes((size_t)qb * kp, 2) + ws_bytes((size_t)qb, 4) +
            ws_bytes((size_t)qb * osegs * ncp, 8) + ws_bytes((size_t)qb * R, 8) +
            ws_bytes((size_t)qb, 4) + ws_bytes((size_t)qb, 8));
  Arena ar(ws);
  __nv_bfloat16* xq = ar.take<__nv_bfloat16>((size_t)qb * kp);
  float* qnorm = ar.take<float>((size_t)qb);
  uint64_t* cand = ar.take<uint64_t>((size_t)qb * osegs * ncp);
  uint64_t* skeys = ar.take<uint64_t>((size_t)qb * R);
  int* over = ar.take<int>((size_t)qb);
  // Shared per-row threshold: exact only when a segment keeps all R keys.
  uint64_t* gthr = (kseg == R && osegs > 1) ? ar.take<uint64_t>((size_t)qb) : nullptr;
  std::vector<int> h_over;
  for (int64_t q0 = 0; q0 < nq; q0 += qb) {
    const int64_t nqb = std::min(qb, nq - q0);
    const float* xb = d_x + q0 * ix->d;
    {
      StageTimer t(ix->ctx, MV_STAGE_FLAT, s);
      if (e4m3) {
        // the query's E4M3 bytes reuse the BF16 query buffer; qnorm holds its scales
        uint8_t* q8 = reinterpret_cast<uint8_t*>(xq);
        launch_to_e4m3(xb, nqb, ix->d, q8, qnorm, nullptr, s);
        launch_umma_topk_e4m3(q8, nqb, qnorm, ix->rows_e4m3.as<uint8_t>(), nb,
                              ix->scales_e4m3.as<float>(), ix->d, ix->metric,
                              ix->norms_e4m3.as<float>(), kseg, nseg, d_filter, gthr, cand,
                              ix->ctx->d_err.as<int>(), s);
      } else {
        launch_to_bf16(xb, nqb, ix->d, xq, qnorm, s);
        launch_umma_topk(xq, nqb, ix->rows_bf16.as<__nv_bfloat16>(), nb, ix->d, ix->metric,
                         nullptr, ix->norms.as<float>(), kseg, nseg, d_filter, gthr, cand,
                         ix->ctx->d_err.as<int>(), s);
      }
    }
    {
      StageTimer t(ix->ctx, MV_STAGE_SELECT, s);
      launch_flat_merge(cand, nqb, osegs, ncp, kseg, R, rerank ? skeys : nullptr, k, qnorm,
                        ix->metric, 0.0f, d_out + q0 * k, d_lab + q0 * k,
                        kseg < R ? over : nullptr, s);
    }
    if (rerank) {
      StageTimer t(ix->ctx, MV_STAGE_RERANK, s);
      RerankArgs r;
      r.q = xb;
      r.nq = nqb;
      r.d = ix->d;
      r.metric = ix->metric;
      r.raw = ix->rows.as<float>();
      r.ids = nullptr;
      r.cand = skeys;
      r.R = R;
      r.k = k;
      r.out_d = d_out + q0 * k;
      r.out_l = d_lab + q0 * k;
      r.ntotal = nb;
      r.err = ix->ctx->d_err.as<int>();
      r.fill_d = 0.0f;  // index_flat.mojo:232-238
      launch_rerank_fast(r, s);
    }
    if (kseg < R) {
      h_over.resize((size_t)nqb);
      d2h(h_over.data(), over, sizeof(int) * nqb, s);
      sync(s);
      std::vector<int64_t> rows;
      for (int64_t i = 0; i < nqb; ++i)
        if (h_over[(size_t)i]) rows.push_back(q0 + i);
      if (!rows.empty()) {
        const int64_t nr = (int64_t)rows.size();
        DevBuf tmp, tws;
        tmp.ensure(ws_bytes((size_t)nr * ix->d, 4) + ws_bytes((size_t)nr * k, 4) +
                   ws_bytes((size_t)nr * k, 8));
        Arena ta(tmp);
        float* tx = ta.take<float>((size_t)nr * ix->d);
        float* td = ta.take<float>((size_t)nr * k);
        int64_t* tl = ta.take<int64_t>((size_t)nr * k);
        for (int64_t i = 0; i < nr; ++i)
          d2d(tx + i * ix->d, d_x + rows[(size_t)i] * ix->d, sizeof(float) * ix->d, s);
        flat_search_exact(ix, tx, nr, k, d_filter, td, tl, tws, s);
        for (int64_t i = 0; i < nr; ++i) {
          d2d(d_out + rows[(size_t)i] * k, td + i * k, sizeof(float) * k, s);
          d2d(d_lab + rows[(size_t)i] * k, tl + i * k, sizeof(int64_t) * k, s);
        }
        sync(s);
        ix->overflow_rows += nr;
      }
    }
  }
}

void flat_search_any(mv_flat* ix, const float* d_x, int64_t nq, int k, const uint8_t* d_filter,
                     const mv_search_params* p, float* d_out, int64_t* d_lab, DevBuf& ws,
                     cudaStream_t s) {
  const int form = p ? p->form : MV_FORM_PLAIN;
  MV_REQUIRE(form == MV_FORM_PLAIN || form == MV_FORM_FAST, MV_ERR_ARG, "unknown search form");
  if (form == MV_FORM_FAST) flat_search_fast(ix, d_x, nq, k, d_filter, p, d_out, d_lab, ws, s);
  else if (p && p->plain_scan) flat_search_exact(ix, d_x, nq, k, d_filter, d_out, d_lab, ws, s);
  else flat_search_plain(ix, d_x, nq, k, d_filter, d_out, d_lab, ws, s);
}

}  // namespace mv

extern "C" {

int32_t mv_flat_create(mv_ctx* ctx, int32_t d, int32_t metric, mv_flat** out) {
  if (!ctx || !out) return MV_ERR_ARG;
  *out = nullptr;
  return guard(ctx, [&] {
    MV_REQUIRE(d > 0 && d <= 65536, MV_ERR_ARG, "dimension must be between 1 and 65536.");
    MV_REQUIRE(metric == MV_METRIC_L2 || metric == MV_METRIC_IP, MV_ERR_ARG, "unknown metric");
    auto ix = std::make_unique<mv_flat>();
    ix->ctx = ctx;
    ix->d = d;
    ix->metric = metric;
    *out = ix.release();
  });
}

int32_t mv_flat_destroy(mv_flat* ix) {
  if (!ix) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    cudaDeviceSynchronize();
    delete ix;
  });
}

int32_t mv_flat_add(mv_flat* ix, const float* x, int64_t n) {
  if (!ix || n < 0 || (n > 0 && !x)) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(ix->mu);
    if (n == 0) return;
    MV_REQUIRE(ix->ntotal + n <= 0xfffffffell, MV_ERR_ARG, "Flat index limited to 2^32 - 2 rows");
    SlotLease lease(ix->ctx);
    cudaStream_t s = lease.stream();
    const int64_t need = ix->ntotal + n;
    if (need > ix->capacity) {  // index_flat.mojo:198-206 capacity doubling
      int64_t cap = std::max<int64_t>(ix->capacity * 2, need);
      DevBuf nb;
      nb.ensure(sizeof(float) * cap * ix->d);
      d2d(nb.p, ix->rows.p, sizeof(float) * ix->ntotal * ix->d, s);
      sync(s);
      std::swap(nb.p, ix->rows.p);
      std::swap(nb.bytes, ix->rows.bytes);
      ix->capacity = cap;
    }
    h2d(ix->rows.as<float>() + ix->ntotal * ix->d, x, sizeof(float) * n * ix->d, s);
    sync(s);
    ix->ntotal = need;
    ix->fast_ready = false;
    ix->e4m3_ready = false;
  });
}

int64_t mv_flat_ntotal(mv_flat* ix) { return ix ? ix->ntotal : -1; }

int32_t mv_flat_search_device(mv_flat* ix, const float* d_x, int64_t nq, int32_t k,
                              const uint8_t* d_filter, const mv_search_params* params,
                              float* d_distances, int64_t* d_labels, void* stream) {
  if (!ix || (nq > 0 && (!d_x || !d_distances || !d_labels))) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    check_search_args(nq, k);
    SlotLease lease(ix->ctx);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : lease.stream();
    lease.use(s);
    flat_search_any(ix, d_x, nq, k, d_filter, params, d_distances, d_labels, lease.slot->ws, s);
    if (!stream) check_kernel_errors(ix->ctx, s);
  });
}

int32_t mv_flat_rerank_device(mv_flat* ix, const float* d_x, int64_t nq, const int64_t* d_cand,
                              int32_t ncand, int32_t k, float* d_distances, int64_t* d_labels,
                              void* stream) {
  if (!ix || nq < 0 || ncand < 0 || (nq > 0 && (!d_x || !d_distances || !d_labels)) ||
      (nq > 0 && ncand > 0 && !d_cand))
    return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    check_search_args(nq, k);
    if (nq == 0) return;
    SlotLease lease(ix->ctx);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : lease.stream();
    lease.use(s);
    DevBuf& ws = lease.slot->ws;
    ws.ensure(ws_bytes((size_t)nq * k, 8));
    Arena ar(ws);
    uint64_t* keys = ar.take<uint64_t>((size_t)nq * k);
    launch_rerank_simd64(d_x, nq, ix->d, ix->rows.as<float>(), ix->ntotal, ix->metric, d_cand,
                         ncand, k, keys, s);
    launch_keys_to_results(keys, nq, k, 0.0f, ix->metric == MV_METRIC_IP, d_distances, d_labels, s);
    if (!stream) check_kernel_errors(ix->ctx, s);
  });
}

int32_t mv_flat_rerank(mv_flat* ix, const float* x, int64_t nq, const int64_t* cand,
                       int32_t ncand, int32_t k, float* distances, int64_t* labels) {
  if (!ix || nq < 0 || ncand < 0 || (nq > 0 && (!x || !distances || !labels)) ||
      (nq > 0 && ncand > 0 && !cand))
    return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    check_search_args(nq, k);
    if (nq == 0) return;
    for (int64_t i = 0; i < nq * (int64_t)ncand; ++i)
      MV_REQUIRE(cand[i] >= -1 && cand[i] < ix->ntotal, MV_ERR_ARG,
                 "candidate ids must be -1 or rows of the index");
    SlotLease lease(ix->ctx);
    cudaStream_t s = lease.stream();
    DevBuf& io = lease.slot->io;
    io.ensure(ws_bytes((size_t)nq * ix->d, 4) + ws_bytes((size_t)nq * ncand + 1, 8) +
              ws_bytes((size_t)nq * k, 8) + ws_bytes((size_t)nq * k, 4) +
              ws_bytes((size_t)nq * k, 8));
    Arena ar(io);
    float* dx = ar.take<float>((size_t)nq * ix->d);
    int64_t* dc = ar.take<int64_t>((size_t)nq * ncand + 1);
    uint64_t* keys = ar.take<uint64_t>((size_t)nq * k);
    float* dd = ar.take<float>((size_t)nq * k);
    int64_t* dl = ar.take<int64_t>((size_t)nq * k);
    h2d(dx, x, sizeof(float) * nq * ix->d, s);
    if (ncand > 0) h2d(dc, cand, sizeof(int64_t) * nq * ncand, s);
    launch_rerank_simd64(dx, nq, ix->d, ix->rows.as<float>(), ix->ntotal, ix->metric, dc, ncand, k,
                         keys, s);
    // index_hnsw.mojo:486-497: ascending, tail 0.0 / -1, IP un-negated
    launch_keys_to_results(keys, nq, k, 0.0f, ix->metric == MV_METRIC_IP, dd, dl, s);
    d2h(distances, dd, sizeof(float) * nq * k, s);
    d2h(labels, dl, sizeof(int64_t) * nq * k, s);
    check_kernel_errors(ix->ctx, s);
  });
}

int32_t mv_flat_search(mv_flat* ix, const float* x, int64_t nq, int32_t k, const uint8_t* filter,
                       const mv_search_params* params, float* distances, int64_t* labels) {
  if (!ix || (nq > 0 && (!x || !distances || !labels))) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    check_search_args(nq, k);
    if (nq == 0) return;
    SlotLease lease(ix->ctx);
    cudaStream_t s = lease.stream();
    DevBuf& io = lease.slot->io;
    const size_t fl = filter ? (size_t)ix->ntotal : 0;
    io.ensure(ws_bytes((size_t)nq * ix->d, 4) + ws_bytes((size_t)nq * k, 4) +
              ws_bytes((size_t)nq * k, 8) + ws_bytes(fl + 1, 1));
    Arena ar(io);
    float* dx = ar.take<float>((size_t)nq * ix->d);
    float* dd = ar.take<float>((size_t)nq * k);
    int64_t* dl = ar.take<int64_t>((size_t)nq * k);
    uint8_t* df = ar.take<uint8_t>(fl + 1);
    h2d(dx, x, sizeof(float) * nq * ix->d, s);
    if (fl) h2d(df, filter, fl, s);
    flat_search_any(ix, dx, nq, k, fl ? df : nullptr, params, dd, dl, lease.slot->ws, s);
    d2h(distances, dd, sizeof(float) * nq * k, s);
    d2h(labels, dl, sizeof(int64_t) * nq * k, s);
    check_kernel_errors(ix->ctx, s);
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// SQ8
// ---------------------------------------------------------------------------
namespace mv {

// Encodes nq queries with the index codec and writes the nq x k shortlist
// keys of the SQ8 scan (index_flat_sq8.mojo:526-583).
void sq8_scan_keys(mv_sq8* ix, const float* d_x, int64_t nq, int kk, const uint8_t* d_filter,
                   uint64_t* out_keys, DevBuf& ws, cudaStream_t s) {
  const bool ip = ix->metric != MV_METRIC_L2;
  const float inv = 1.0f / ix->scale;
  const float scale_sq = ix->scale * ix->scale;
  const int64_t nb = ix->ntotal;
  int64_t cb = (int64_t)(1024ll * 1024 * 1024 / 4) / std::max<int64_t>(nq, 1);
  cb = std::max<int64_t>(64, (cb / 64) * 64);
  cb = std::min(cb, std::max<int64_t>(nb, 1));
  ws.ensure(ws_bytes((size_t)nq * ix->dpad, 1) + ws_bytes(nq, 4) + ws_bytes((size_t)nq * cb, 4) +
            ws_bytes((size_t)nq * kk, 8));
  Arena ar(ws);
  uint8_t* qc = ar.take<uint8_t>((size_t)nq * ix->dpad);
  uint32_t* qn = ar.take<uint32_t>(nq);
  float* dmat = ar.take<float>((size_t)nq * cb);
  uint64_t* tmp = ar.take<uint64_t>((size_t)nq * kk);
  launch_sq8_encode(d_x, nq, ix->d, ix->dpad, ip ? 0.0f : ix->gmin, inv, ip, qc, qn, s);
  uint64_t* cur = out_keys;
  uint64_t* nxt = tmp;
  // Chunks alternate between the two key buffers; pick the start so that
  // the last chunk writes out_keys.
  int64_t nchunks = (nb + cb - 1) / cb;
  if (nchunks % 2 == 1) std::swap(cur, nxt);
  bool first = true;
  for (int64_t c0 = 0; c0 < nb; c0 += cb) {
    const int64_t nc = std::min(cb, nb - c0);
    launch_sq8_matrix(qc, qn, nq, ix->codes.as<uint8_t>() + c0 * ix->dpad,
                      ix->norms.as<uint32_t>() + c0, nc, ix->dpad, ip, scale_sq, dmat, nc, s);
    launch_select_rows(dmat, nq, nc, nc, c0, kk, first ? nullptr : cur, nxt, d_filter, s);
    std::swap(cur, nxt);
    first = false;
  }
}

__global__ void k_keys_to_cand(const uint64_t* __restrict__ keys, int64_t n, int64_t* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = keys[i] == ~0ull ? -1 : (int64_t)(uint32_t)keys[i];
}

// The tensor-core SQ8 scan is exact when every BF16 product and FP32
// partial sum is an integer below 2^24: L2 (u8 codes) needs
// 2 * d * 255^2 < 2^24 (d <= 129), IP (s8 codes) d * 127^2 < 2^24
// (d <= 1040).
bool sq8_tensor_exact(const mv_sq8* ix) {
  if (umma_kpad(ix->d) > UMMA_TOPK_MAX_K) return false;
  if (ix->metric == MV_METRIC_L2) return 2ll * ix->d * 255 * 255 < (1ll << 24);
  return (int64_t)ix->d * 127 * 127 < (1ll << 24);
}

void ensure_sq8_fast(mv_sq8* ix, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(ix->fast_mu);
  if (ix->fast_ready) return;
  const int kp = umma_kpad(ix->d);
  ix->codes_bf16.ensure((size_t)ix->ntotal * kp * 2);
  ix->fnorms.ensure((size_t)ix->ntotal * 4);
  launch_sq8_codes_to_bf16(ix->codes.as<uint8_t>(), ix->ntotal, ix->d, ix->dpad, kp,
                           ix->metric != MV_METRIC_L2, ix->norms.as<uint32_t>(),
                           ix->codes_bf16.as<__nv_bfloat16>(), ix->fnorms.as<float>(), s);
  sync(s);
  ix->fast_ready = true;
}

// Shortlist keys of the SQ8 scan (nq x R canonical (distance, row) keys,
// the same set and order as sq8_scan_keys) from the tensor-core GEMM over
// BF16 codes; queries flagged by the merge are rescanned with the exact
// integer kernel.
void sq8_tensor_keys(mv_sq8* ix, const float* d_x, int64_t nq, int R, const uint8_t* d_filter,
                     uint64_t* out_keys, DevBuf& ws, cudaStream_t s) {
  ensure_sq8_fast(ix, s);
  const bool ip = ix->metric != MV_METRIC_L2;
  const int64_t nb = ix->ntotal;
  const int kp = umma_kpad(ix->d);
  const int kseg = std::min(R + 8, UMMA_TOPK_MAX);  // a margin for distance ties
  const int ncp = next_pow2(kseg);
  int nseg = umma_topk_nseg(nq, nb, ix->d, kseg, ix->ctx->num_sms);
  const int groups = umma_topk_groups(ix->d, kseg);
  if (kseg < R + 8) {  // as for the flat scan: independent of the batch
    const int64_t nct = (nb + 127) / 128;
    nseg = (int)std::min<int64_t>((R + 15) / 16 / groups + 1, std::max<int64_t>(1, nct));
  }
  const int osegs = nseg * groups;
  ws.ensure(ws_bytes((size_t)nq * ix->dpad, 1) + ws_bytes((size_t)nq, 4) +
            ws_bytes((size_t)nq * kp, 2) + ws_bytes((size_t)nq * osegs * ncp, 8) +
            ws_bytes((size_t)nq, 4));
  Arena ar(ws);
  uint8_t* qc = ar.take<uint8_t>((size_t)nq * ix->dpad);
  uint32_t* qn = ar.take<uint32_t>((size_t)nq);
  __nv_bfloat16* xq = ar.take<__nv_bfloat16>((size_t)nq * kp);
  uint64_t* cand = ar.take<uint64_t>((size_t)nq * osegs * ncp);
  int* flag = ar.take<int>((size_t)nq);
  launch_sq8_encode(d_x, nq, ix->d, ix->dpad, ip ? 0.0f : ix->gmin, 1.0f / ix->scale, ip, qc, qn, s);
  launch_sq8_codes_to_bf16(qc, nq, ix->d, ix->dpad, kp, ip, qn, xq, nullptr, s);
  {
    StageTimer t(ix->ctx, MV_STAGE_FLAT, s);
    launch_umma_topk(xq, nq, ix->codes_bf16.as<__nv_bfloat16>(), nb, ix->d, ix->metric, nullptr,
                     ix->fnorms.as<float>(), kseg, nseg, d_filter, nullptr, cand,
                     ix->ctx->d_err.as<int>(), s);
  }
  {
    StageTimer t(ix->ctx, MV_STAGE_SELECT, s);
    launch_sq8_merge(cand, nq, osegs, ncp, kseg, R, qn, ip, ix->scale * ix->scale, out_keys, flag,
                     s);
  }
  std::vector<int> h_flag((size_t)nq);
  d2h(h_flag.data(), flag, sizeof(int) * nq, s);
  sync(s);
  std::vector<int64_t> rows;
  for (int64_t i = 0; i < nq; ++i)
    if (h_flag[(size_t)i]) rows.push_back(i);
  if (rows.empty()) return;
  const int64_t nr = (int64_t)rows.size();
  DevBuf tmp, tws;
  tmp.ensure(ws_bytes((size_t)nr * ix->d, 4) + ws_bytes((size_t)nr * R, 8));
  Arena ta(tmp);
  float* tx = ta.take<float>((size_t)nr * ix->d);
  uint64_t* tk = ta.take<uint64_t>((size_t)nr * R);
  for (int64_t i = 0; i < nr; ++i)
    d2d(tx + i * ix->d, d_x + rows[(size_t)i] * ix->d, sizeof(float) * ix->d, s);
  sq8_scan_keys(ix, tx, nr, R, d_filter, tk, tws, s);
  for (int64_t i = 0; i < nr; ++i)
    d2d(out_keys + rows[(size_t)i] * R, tk + i * R, sizeof(uint64_t) * R, s);
  sync(s);
  ix->fallback_rows += nr;
}

void sq8_search_impl(mv_sq8* ix, const float* d_x, int64_t nq, int k, int rerank_factor,
                     const uint8_t* d_filter, float* d_out, int64_t* d_lab, DevBuf& ws,
                     cudaStream_t s, bool tensor = false) {
  if (nq == 0) return;
  // The tensor-core scan returns the same keys as the integer scan; it is
  // used when asked for and exact for this dimension and metric.
  auto keys_of = [&](int R, uint64_t* out) {
    if (tensor && sq8_tensor_exact(ix)) sq8_tensor_keys(ix, d_x, nq, R, d_filter, out, ws, s);
    else sq8_scan_keys(ix, d_x, nq, R, d_filter, out, ws, s);
  };
  const bool ip = ix->metric != MV_METRIC_L2;
  if (ix->ntotal == 0) {
    launch_fill(d_out, d_lab, nq * k, 0.0f, s);
    return;
  }
  if (rerank_factor <= 0) {
    DevBuf keys;
    keys.ensure(sizeof(uint64_t) * nq * k);
    keys_of(k, keys.as<uint64_t>());
    launch_keys_to_results(keys.as<uint64_t>(), nq, k, 0.0f, ip, d_out, d_lab, s);  // :595-602
    sync(s);
    return;
  }
  const int kk = (int)std::min<int64_t>((int64_t)k * rerank_factor, 2048);
  DevBuf keys, cand, fk;
  keys.ensure(sizeof(uint64_t) * nq * kk);
  cand.ensure(sizeof(int64_t) * nq * kk);
  fk.ensure(sizeof(uint64_t) * nq * k);
  keys_of(kk, keys.as<uint64_t>());
  k_keys_to_cand<<<(unsigned)((nq * kk + 255) / 256), 256, 0, s>>>(keys.as<uint64_t>(), nq * kk,
                                                                  cand.as<int64_t>());
  count_launch();
  launch_rerank_simd64(d_x, nq, ix->d, ix->f32.as<float>(), ix->ntotal, ix->metric,
                       cand.as<int64_t>(), kk, k, fk.as<uint64_t>(), s);
  launch_keys_to_results(fk.as<uint64_t>(), nq, k, 0.0f, ip, d_out, d_lab, s);
  sync(s);
}

}  // namespace mv

extern "C" {

int32_t mv_sq8_create(mv_ctx* ctx, int32_t d, int32_t metric, mv_sq8** out) {
  if (!ctx || !out) return MV_ERR_ARG;
  *out = nullptr;
  return guard(ctx, [&] {
    MV_REQUIRE(d > 0 && d <= 65536, MV_ERR_ARG, "dimension must be between 1 and 65536.");
    MV_REQUIRE(metric == MV_METRIC_L2 || metric == MV_METRIC_IP, MV_ERR_ARG, "unknown metric");
    auto ix = std::make_unique<mv_sq8>();
    ix->ctx = ctx;
    ix->d = d;
    ix->dpad = (d + 15) / 16 * 16;
    ix->metric = metric;
    ix->gmin = std::numeric_limits<float>::max();   // index_flat_sq8.mojo:311-313
    ix->gmax = -std::numeric_limits<float>::max();
    ix->scale = 1.0f;
    *out = ix.release();
  });
}

int32_t mv_sq8_destroy(mv_sq8* ix) {
  if (!ix) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    cudaDeviceSynchronize();
    delete ix;
  });
}

int32_t mv_sq8_add(mv_sq8* ix, const float* x, int64_t n) {
  if (!ix || n < 0 || (n > 0 && !x)) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(ix->mu);
    if (n == 0) return;  // :373-374
    MV_REQUIRE(ix->ntotal + n <= 0xfffffffell, MV_ERR_ARG, "SQ8 index limited to 2^32 - 2 rows");
    SlotLease lease(ix->ctx);
    cudaStream_t s = lease.stream();
    const int d = ix->d, dp = ix->dpad;
    const int64_t need = ix->ntotal + n;
    if (need > ix->capacity) {  // :376-394
      int64_t cap = std::max<int64_t>(ix->capacity * 2, need);
      DevBuf f, c, nm;
      f.ensure(sizeof(float) * cap * d);
      c.ensure((size_t)cap * dp);
      nm.ensure(sizeof(uint32_t) * cap);
      d2d(f.p, ix->f32.p, sizeof(float) * ix->ntotal * d, s);
      d2d(c.p, ix->codes.p, (size_t)ix->ntotal * dp, s);
      d2d(nm.p, ix->norms.p, sizeof(uint32_t) * ix->ntotal, s);
      sync(s);
      std::swap(f.p, ix->f32.p);
      std::swap(f.bytes, ix->f32.bytes);
      std::swap(c.p, ix->codes.p);
      std::swap(c.bytes, ix->codes.bytes);
      std::swap(nm.p, ix->norms.p);
      std::swap(nm.bytes, ix->norms.bytes);
      ix->capacity = cap;
    }
    float* newrows = ix->f32.as<float>() + ix->ntotal * d;
    h2d(newrows, x, sizeof(float) * n * d, s);
    DevBuf mm;
    mm.ensure(8);
    launch_minmax(newrows, n * d, mm.as<float>(), s);  // :397-402
    float bminmax[2];
    d2h(bminmax, mm.p, 8, s);
    sync(s);
    bool requant = false;  // :404-410
    if (bminmax[0] < ix->gmin) {
      ix->gmin = bminmax[0];
      requant = true;
    }
    if (bminmax[1] > ix->gmax) {
      ix->gmax = bminmax[1];
      requant = true;
    }
    const bool sym = ix->metric != MV_METRIC_L2;
    if (!sym) {  // :412-421
      ix->scale = (ix->gmax == ix->gmin) ? 1.0f : (ix->gmax - ix->gmin) / 255.0f;
    } else {
      float max_abs = std::max(std::fabs(ix->gmin), std::fabs(ix->gmax));
      ix->scale = max_abs > 0.0f ? max_abs / 127.0f : 1.0f;
    }
    const float inv = 1.0f / ix->scale;  // :423
    const float mn = sym ? 0.0f : ix->gmin;
    if (requant && ix->ntotal > 0)  // :426-446
      launch_sq8_encode(ix->f32.as<float>(), ix->ntotal, d, dp, mn, inv, sym, ix->codes.as<uint8_t>(),
                        ix->norms.as<uint32_t>(), s);
    launch_sq8_encode(newrows, n, d, dp, mn, inv, sym, ix->codes.as<uint8_t>() + ix->ntotal * dp,
                      ix->norms.as<uint32_t>() + ix->ntotal, s);
    sync(s);
    ix->ntotal = need;
    ix->fast_ready = false;
  });
}

int32_t mv_sq8_params(mv_sq8* ix, float* out3) {
  if (!ix || !out3) return MV_ERR_ARG;
  out3[0] = ix->gmin;
  out3[1] = ix->gmax;
  out3[2] = ix->scale;
  return MV_OK;
}

int64_t mv_sq8_ntotal(mv_sq8* ix) { return ix ? ix->ntotal : -1; }

int32_t mv_sq8_get_codes(mv_sq8* ix, uint8_t* codes, uint32_t* norms) {
  if (!ix) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(ix->mu);
    if (ix->ntotal == 0) return;
    if (codes)
      MV_CHECK_CUDA(cudaMemcpy2D(codes, ix->d, ix->codes.p, ix->dpad, ix->d, ix->ntotal,
                                 cudaMemcpyDeviceToHost));
    if (norms)
      MV_CHECK_CUDA(cudaMemcpy(norms, ix->norms.p, sizeof(uint32_t) * ix->ntotal, cudaMemcpyDeviceToHost));
  });
}

static int32_t sq8_search_host(mv_sq8* ix, const float* x, int64_t nq, int32_t k,
                               const uint8_t* filter, int rerank_factor, float* distances,
                               int64_t* labels, bool tensor = false) {
  if (!ix || (nq > 0 && (!x || !distances || !labels))) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    check_search_args(nq, k);
    if (nq == 0) return;
    SlotLease lease(ix->ctx);
    cudaStream_t s = lease.stream();
    DevBuf& io = lease.slot->io;
    const size_t fl = filter ? (size_t)ix->ntotal : 0;
    io.ensure(ws_bytes((size_t)nq * ix->d, 4) + ws_bytes((size_t)nq * k, 4) +
              ws_bytes((size_t)nq * k, 8) + ws_bytes(fl + 1, 1));
    Arena ar(io);
    float* dx = ar.take<float>((size_t)nq * ix->d);
    float* dd = ar.take<float>((size_t)nq * k);
    int64_t* dl = ar.take<int64_t>((size_t)nq * k);
    uint8_t* df = ar.take<uint8_t>(fl + 1);
    h2d(dx, x, sizeof(float) * nq * ix->d, s);
    if (fl) h2d(df, filter, fl, s);
    sq8_search_impl(ix, dx, nq, k, rerank_factor, fl ? df : nullptr, dd, dl, lease.slot->ws, s,
                    tensor);
    d2h(distances, dd, sizeof(float) * nq * k, s);
    d2h(labels, dl, sizeof(int64_t) * nq * k, s);
    check_kernel_errors(ix->ctx, s);
  });
}

// The plain SQ8 entry points take the tensor-core keys where they are exact
// (they equal the integer scan's bit for bit), the integer scan elsewhere.
int32_t mv_sq8_search(mv_sq8* ix, const float* x, int64_t nq, int32_t k, const uint8_t* filter,
                      float* distances, int64_t* labels) {
  return sq8_search_host(ix, x, nq, k, filter, 0, distances, labels, true);
}

int32_t mv_sq8_search_rerank(mv_sq8* ix, const float* x, int64_t nq, int32_t k,
                             int32_t rerank_factor, float* distances, int64_t* labels) {
  if (rerank_factor < 1) return MV_ERR_ARG;
  return sq8_search_host(ix, x, nq, k, nullptr, rerank_factor, distances, labels, true);
}

int32_t mv_sq8_search_device(mv_sq8* ix, const float* d_x, int64_t nq, int32_t k,
                             const uint8_t* d_filter, int32_t rerank_factor,
                             const mv_search_params* params, float* d_distances,
                             int64_t* d_labels, void* stream) {
  if (!ix || rerank_factor < 0 || (nq > 0 && (!d_x || !d_distances || !d_labels)))
    return MV_ERR_ARG;
  const int form = params ? params->form : MV_FORM_PLAIN;
  if (form != MV_FORM_PLAIN && form != MV_FORM_FAST) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    check_search_args(nq, k);
    SlotLease lease(ix->ctx);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : lease.stream();
    lease.use(s);
    sq8_search_impl(ix, d_x, nq, k, rerank_factor, d_filter, d_distances, d_labels,
                    lease.slot->ws, s, form == MV_FORM_FAST || !(params && params->plain_scan));
    if (!stream) check_kernel_errors(ix->ctx, s);
  });
}

int32_t mv_sq8_search_ex(mv_sq8* ix, const float* x, int64_t nq, int32_t k,
                         const uint8_t* filter, int32_t rerank_factor,
                         const mv_search_params* params, float* distances, int64_t* labels) {
  if (rerank_factor < 0) return MV_ERR_ARG;
  const int form = params ? params->form : MV_FORM_PLAIN;
  if (form != MV_FORM_PLAIN && form != MV_FORM_FAST) return MV_ERR_ARG;
  return sq8_search_host(ix, x, nq, k, filter, rerank_factor, distances, labels,
                         form == MV_FORM_FAST || !(params && params->plain_scan));
}

// ---------------------------------------------------------------------------
// primitives
// ---------------------------------------------------------------------------
int32_t mv_kmeans_train(mv_ctx* ctx, const float* x, int64_t n, int32_t d, int32_t k,
                        int32_t niter, float* centroids, int64_t* assignments) {
  if (!ctx || n < 0 || (n > 0 && (!x || !centroids)) || d <= 0 || k <= 0) return MV_ERR_ARG;
  return guard(ctx, [&] {
    if (n == 0) return;  // kmeans.mojo:62
    SlotLease lease(ctx);
    cudaStream_t s = lease.stream();
    DevBuf dx, dc, da, scratch;
    dx.ensure(sizeof(float) * n * d);
    dc.ensure(sizeof(float) * k * d);
    da.ensure(sizeof(int32_t) * n);
    h2d(dx.p, x, sizeof(float) * n * d, s);
    kmeans_train_device(dx.as<float>(), n, d, k, niter, 1, dc.as<float>(), da.as<int32_t>(),
                        scratch, s);
    d2h(centroids, dc.p, sizeof(float) * k * d, s);
    if (assignments) {
      DevBuf a64;
      a64.ensure(sizeof(int64_t) * n);
      launch_i32_to_i64(da.as<int32_t>(), n, a64.as<int64_t>(), s);
      d2h(assignments, a64.p, sizeof(int64_t) * n, s);
      sync(s);
    }
    sync(s);
  });
}

int32_t mv_kmeans_train_ex(mv_ctx* ctx, const float* x, int64_t n, int32_t d, int32_t k,
                           int32_t niter, const mv_search_params* params, float* centroids,
                           int64_t* assignments, double* objective) {
  if (!ctx || n < 0 || (n > 0 && (!x || !centroids)) || d <= 0 || k <= 0 || niter < 0)
    return MV_ERR_ARG;
  const int form = params ? params->form : MV_FORM_PLAIN;
  if (form != MV_FORM_PLAIN && form != MV_FORM_FAST) return MV_ERR_ARG;
  return guard(ctx, [&] {
    if (n == 0) return;  // kmeans.mojo:62
    SlotLease lease(ctx);
    cudaStream_t s = lease.stream();
    DevBuf dx, dc, da, scratch, dobj;
    dx.ensure(sizeof(float) * n * d);
    dc.ensure(sizeof(float) * k * d);
    da.ensure(sizeof(int32_t) * n);
    if (objective) dobj.ensure(sizeof(double) * (niter + 1));
    h2d(dx.p, x, sizeof(float) * n * d, s);
    double* d_obj = objective ? dobj.as<double>() : nullptr;
    {
      StageTimer t(ctx, MV_STAGE_COARSE, s);
      if (form == MV_FORM_FAST)
        kmeans_train_fast(dx.as<float>(), n, d, k, niter, dc.as<float>(), da.as<int32_t>(),
                          scratch, ctx, s, d_obj);
      else
        kmeans_train_device(dx.as<float>(), n, d, k, niter, 1, dc.as<float>(), da.as<int32_t>(),
                            scratch, s, d_obj);
    }
    d2h(centroids, dc.p, sizeof(float) * k * d, s);
    if (objective) d2h(objective, d_obj, sizeof(double) * (niter + 1), s);
    if (assignments) {
      DevBuf a64;
      a64.ensure(sizeof(int64_t) * n);
      launch_i32_to_i64(da.as<int32_t>(), n, a64.as<int64_t>(), s);
      d2h(assignments, a64.p, sizeof(int64_t) * n, s);
      sync(s);
    }
    check_kernel_errors(ctx, s);
  });
}

int32_t mv_pq_train(mv_ctx* ctx, const float* x, int64_t n, int32_t d, int32_t M, int32_t niter,
                    float* pq) {
  if (!ctx || n <= 0 || !x || !pq || d <= 0 || M <= 0 || d % M != 0) return MV_ERR_ARG;
  return guard(ctx, [&] {
    SlotLease lease(ctx);
    cudaStream_t s = lease.stream();
    DevBuf dx, dp, work, scratch;
    dx.ensure(sizeof(float) * n * d);
    dp.ensure(sizeof(float) * 256 * d);
    h2d(dx.p, x, sizeof(float) * n * d, s);
    pq_train_device(dx.as<float>(), n, d, M, niter, dp.as<float>(), work, scratch, s);
    d2h(pq, dp.p, sizeof(float) * 256 * d, s);
    sync(s);
  });
}

int32_t mv_pq_encode(mv_ctx* ctx, const float* pq, int32_t d, int32_t M, const float* x, int64_t n,
                     uint8_t* codes) {
  if (!ctx || !pq || d <= 0 || M <= 0 || d % M != 0 || n < 0 || (n > 0 && (!x || !codes)))
    return MV_ERR_ARG;
  return guard(ctx, [&] {
    if (n == 0) return;
    SlotLease lease(ctx);
    cudaStream_t s = lease.stream();
    DevBuf dx, dp, dc;
    dx.ensure(sizeof(float) * n * d);
    dp.ensure(sizeof(float) * 256 * d);
    dc.ensure((size_t)n * M);
    h2d(dx.p, x, sizeof(float) * n * d, s);
    h2d(dp.p, pq, sizeof(float) * 256 * d, s);
    launch_pq_encode(dx.as<float>(), n, d, M, dp.as<float>(), dc.as<uint8_t>(), s);
    d2h(codes, dc.p, (size_t)n * M, s);
    sync(s);
  });
}

int32_t mv_pq_distance_tables(mv_ctx* ctx, const float* pq, int32_t d, int32_t M, const float* x,
                              int64_t nq, int32_t metric, float* tables) {
  if (!ctx || !pq || d <= 0 || M <= 0 || d % M != 0 || nq < 0 || (nq > 0 && (!x || !tables)))
    return MV_ERR_ARG;
  return guard(ctx, [&] {
    if (nq == 0) return;
    SlotLease lease(ctx);
    cudaStream_t s = lease.stream();
    DevBuf dx, dp, dt;
    dx.ensure(sizeof(float) * nq * d);
    dp.ensure(sizeof(float) * 256 * d);
    dt.ensure(sizeof(float) * nq * M * 256);
    h2d(dx.p, x, sizeof(float) * nq * d, s);
    h2d(dp.p, pq, sizeof(float) * 256 * d, s);
    launch_pq_tables(dx.as<float>(), nq, d, M, dp.as<float>(), metric, dt.as<float>(), s);
    d2h(tables, dt.p, sizeof(float) * nq * M * 256, s);
    sync(s);
  });
}

int32_t mv_sq8_encode(mv_ctx* ctx, const float* x, int64_t n, int32_t d, float minimum,
                      float inverse_scale, int32_t symmetric, uint8_t* codes, uint32_t* norms) {
  if (!ctx || d <= 0 || n < 0 || (n > 0 && (!x || !codes || !norms))) return MV_ERR_ARG;
  return guard(ctx, [&] {
    if (n == 0) return;
    SlotLease lease(ctx);
    cudaStream_t s = lease.stream();
    const int dp = (d + 15) / 16 * 16;
    DevBuf dx, dc, dn;
    dx.ensure(sizeof(float) * n * d);
    dc.ensure((size_t)n * dp);
    dn.ensure(sizeof(uint32_t) * n);
    h2d(dx.p, x, sizeof(float) * n * d, s);
    launch_sq8_encode(dx.as<float>(), n, d, dp, minimum, inverse_scale, symmetric != 0,
                      dc.as<uint8_t>(), dn.as<uint32_t>(), s);
    MV_CHECK_CUDA(cudaMemcpy2DAsync(codes, d, dc.p, dp, d, n, cudaMemcpyDeviceToHost, s));
    d2h(norms, dn.p, sizeof(uint32_t) * n, s);
    sync(s);
  });
}

int32_t mv_distance_matrix(mv_ctx* ctx, const float* x, int64_t nx, const float* y, int64_t ny,
                           int32_t d, int32_t metric, int32_t precision, float* out) {
  if (!ctx || d <= 0 || nx < 0 || ny < 0 || (nx > 0 && ny > 0 && (!x || !y || !out)))
    return MV_ERR_ARG;
  return guard(ctx, [&] {
    MV_REQUIRE(metric == MV_METRIC_L2 || metric == MV_METRIC_IP, MV_ERR_ARG, "unknown metric");
    MV_REQUIRE(precision == 0 || precision == 1, MV_ERR_ARG, "precision must be 0 or 1");
    if (nx == 0 || ny == 0) return;
    SlotLease lease(ctx);
    cudaStream_t s = lease.stream();
    DevBuf dx, dy, dout, bx, by, nxb, nyb;
    dx.ensure(sizeof(float) * nx * d);
    dy.ensure(sizeof(float) * ny * d);
    dout.ensure(sizeof(float) * nx * ny);
    h2d(dx.p, x, sizeof(float) * nx * d, s);
    h2d(dy.p, y, sizeof(float) * ny * d, s);
    if (precision == 0) {
      launch_exact_matrix(metric == MV_METRIC_L2 ? KIND_L2_SIMD8 : KIND_IP_SIMD8, dx.as<float>(), nx,
                          d, dy.as<float>(), ny, d, d, dout.as<float>(), ny, s);
    } else {
      const int kp = umma_kpad(d);
      bx.ensure(sizeof(uint16_t) * nx * kp);
      by.ensure(sizeof(uint16_t) * ny * kp);
      nxb.ensure(sizeof(float) * nx);
      nyb.ensure(sizeof(float) * ny);
      launch_to_bf16(dx.as<float>(), nx, d, bx.as<__nv_bfloat16>(), nxb.as<float>(), s);
      launch_to_bf16(dy.as<float>(), ny, d, by.as<__nv_bfloat16>(), nyb.as<float>(), s);
      launch_umma_dist(EPI_MATRIX, bx.as<__nv_bfloat16>(), nx, by.as<__nv_bfloat16>(), ny, d, metric,
                       nxb.as<float>(), nyb.as<float>(), dout.as<float>(), ny, nullptr,
                       ctx->d_err.as<int>(), ctx->num_sms, s);
    }
    d2h(out, dout.p, sizeof(float) * nx * ny, s);
    check_kernel_errors(ctx, s);
  });
}

int32_t mv_normalize(mv_ctx* ctx, const float* x, int64_t n, int32_t d, float* out) {
  if (!ctx || d <= 0 || n < 0 || (n > 0 && (!x || !out))) return MV_ERR_ARG;
  return guard(ctx, [&] {
    if (n == 0) return;
    SlotLease lease(ctx);
    cudaStream_t s = lease.stream();
    DevBuf dx, dy, bad;
    dx.ensure(sizeof(float) * n * d);
    dy.ensure(sizeof(float) * n * d);
    bad.ensure(4);
    MV_CHECK_CUDA(cudaMemsetAsync(bad.p, 0, 4, s));
    h2d(dx.p, x, sizeof(float) * n * d, s);
    launch_normalize(dx.as<float>(), n, d, dy.as<float>(), bad.as<int32_t>(), s);
    int32_t hb = 0;
    d2h(&hb, bad.p, 4, s);
    sync(s);
    MV_REQUIRE(hb != 1, MV_ERR_ARG, "Vector components must be finite.");
    MV_REQUIRE(hb != 2, MV_ERR_ARG, "Cosine embeddings must be non-zero vectors.");
    d2h(out, dy.p, sizeof(float) * n * d, s);
    sync(s);
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched fast IVF-PQ: plan with per-query nprobe / k, a persistent scan,
// CUDA graphs per batch size and a tuner for the launch shapes.
// ---------------------------------------------------------------------------
struct mv_ivfpq_plan {
  mv_ivfpq* ix = nullptr;
  int64_t max_nq = 0;
  int nprobe_max = 1, kmax = 1;
  mv_search_params params{};
  cudaStream_t stream = nullptr;
  mv::DevBuf x, nprobe_q, k_q, order, out_d, out_l, counter, ws;
  mv::FastBatch cfg;
  std::map<int64_t, cudaGraphExec_t> graphs;   // one per batch size
  std::map<int64_t, int64_t> graph_kernels;    // kernels per replay
  std::mutex mu;
  ~mv_ivfpq_plan() {
    for (auto& g : graphs) cudaGraphExecDestroy(g.second);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace mv {

FastBatch plan_batch(mv_ivfpq_plan* pl) {
  FastBatch b = pl->cfg;
  b.nprobe_q = pl->nprobe_q.as<int32_t>();
  b.k_q = pl->k_q.as<int32_t>();
  b.order = pl->order.as<int32_t>();
  b.counter = pl->counter.as<int>();
  return b;
}

void plan_enqueue(mv_ivfpq_plan* pl, int64_t nq, cudaStream_t s) {
  const FastBatch b = plan_batch(pl);
  ivfpq_search_fast(pl->ix, pl->x.as<float>(), nq, pl->kmax, pl->nprobe_max, &pl->params,
                    pl->out_d.as<float>(), pl->out_l.as<int64_t>(), pl->ws, s, &b);
}

void plan_drop_graphs(mv_ivfpq_plan* pl) {
  for (auto& g : pl->graphs) cudaGraphExecDestroy(g.second);
  pl->graphs.clear();
  pl->graph_kernels.clear();
}

// Runs the batch; with use_graph the enqueue is captured once per batch size
// (after a direct run that sizes the workspace and raises the kernels'
// shared-memory limits) and replayed.
void plan_run(mv_ivfpq_plan* pl, int64_t nq, cudaStream_t s, bool use_graph) {
  mv_ivfpq* ix = pl->ix;
  ensure_fast(ix, s);
  if (!use_graph) {
    plan_enqueue(pl, nq, s);
    return;
  }
  auto it = pl->graphs.find(nq);
  if (it == pl->graphs.end()) {
    plan_enqueue(pl, nq, s);
    sync(s);
    const bool prof = ix->ctx->profile.exchange(false);  // no event nodes in the graph
    const int64_t l0 = ix->ctx->launches.load();
    cudaGraph_t g = nullptr;
    MV_CHECK_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      plan_enqueue(pl, nq, s);
    } catch (...) {
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      ix->ctx->profile.store(prof);
      throw;
    }
    MV_CHECK_CUDA(cudaStreamEndCapture(s, &g));
    ix->ctx->profile.store(prof);
    cudaGraphExec_t exec = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    MV_CHECK_CUDA(e);
    it = pl->graphs.emplace(nq, exec).first;
    pl->graph_kernels[nq] = ix->ctx->launches.load() - l0;
    ix->ctx->launches.fetch_sub(pl->graph_kernels[nq]);  // counted again per replay
  }
  MV_CHECK_CUDA(cudaGraphLaunch(it->second, s));
  ix->ctx->launches.fetch_add(pl->graph_kernels[nq]);
}

// Tuner: coordinate descent over the coarse method (fused top-k GEMM or
// distance matrix, where both apply), the scan's threads per CTA and its
// persistent grid, each candidate timed with CUDA events on the plan's own
// batch (median of 3 after a warm-up). Returns the best time in ms.
float plan_tune(mv_ivfpq_plan* pl, int64_t nq, cudaStream_t s) {
  mv_ivfpq* ix = pl->ix;
  ensure_fast(ix, s);
  cudaEvent_t a, b;
  MV_CHECK_CUDA(cudaEventCreate(&a));
  MV_CHECK_CUDA(cudaEventCreate(&b));
  auto time_cfg = [&](const FastBatch& c) -> float {
    pl->cfg = c;
    plan_enqueue(pl, nq, s);
    float t[3];
    for (int r = 0; r < 3; ++r) {
      cudaEventRecord(a, s);
      plan_enqueue(pl, nq, s);
      cudaEventRecord(b, s);
      MV_CHECK_CUDA(cudaEventSynchronize(b));
      cudaEventElapsedTime(&t[r], a, b);
    }
    std::sort(t, t + 3);
    return t[1];
  };
  FastBatch best = pl->cfg;
  float best_ms = time_cfg(best);
  auto consider = [&](FastBatch c) {
    const float ms = time_cfg(c);
    if (ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  };
  const int nc = std::min(ix->nlist, pl->nprobe_max + std::max(8, pl->nprobe_max / 4));
  if (nc <= 64 && !pl->params.coarse_fp32) {
    FastBatch c = best;
    c.coarse_matrix = !c.coarse_matrix;
    consider(c);
  }
  for (int nt : {128, 256, 512}) {
    if (nt == best.scan_threads) continue;
    FastBatch c = best;
    c.scan_threads = nt;
    consider(c);
  }
  for (int cps : {0, 2, 4, 8}) {
    if (cps == best.scan_ctas_per_sm) continue;
    FastBatch c = best;
    c.scan_ctas_per_sm = cps;
    consider(c);
  }
  pl->cfg = best;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  plan_drop_graphs(pl);
  return best_ms;
}

// Host-side per-query parameters -> plan buffers, and the scan order:
// queries by decreasing nprobe (ties by index), so the persistent grid
// starts the longest scans first.
void plan_set_queries(mv_ivfpq_plan* pl, const float* x, int64_t nq, const int32_t* nprobe,
                      const int32_t* k, cudaStream_t s) {
  MV_REQUIRE(nq >= 0 && nq <= pl->max_nq, MV_ERR_ARG, "batch larger than the plan");
  std::vector<int32_t> np(nq), kk(nq), ord(nq);
  for (int64_t i = 0; i < nq; ++i) {
    np[i] = nprobe ? std::min(nprobe[i], pl->ix->nlist) : pl->nprobe_max;  // at most nlist lists
    kk[i] = k ? k[i] : pl->kmax;
    MV_REQUIRE(np[i] >= 1 && np[i] <= pl->nprobe_max, MV_ERR_ARG,
               "per-query nprobe must be between 1 and the plan's nprobe");
    MV_REQUIRE(kk[i] >= 1 && kk[i] <= pl->kmax, MV_ERR_ARG,
               "per-query k must be between 1 and the plan's k");
    ord[i] = (int32_t)i;
  }
  std::stable_sort(ord.begin(), ord.end(), [&](int32_t p, int32_t q) { return np[p] > np[q]; });
  if (x) h2d(pl->x.p, x, sizeof(float) * nq * pl->ix->d, s);
  h2d(pl->nprobe_q.p, np.data(), sizeof(int32_t) * nq, s);
  h2d(pl->k_q.p, kk.data(), sizeof(int32_t) * nq, s);
  h2d(pl->order.p, ord.data(), sizeof(int32_t) * nq, s);
  sync(s);  // the host vectors go out of scope
}

}  // namespace mv

extern "C" {

int32_t mv_ivfpq_plan_create(mv_ivfpq* ix, int64_t max_nq, int32_t nprobe_max, int32_t kmax,
                             const mv_search_params* params, mv_ivfpq_plan** out) {
  if (!ix || !out || max_nq <= 0 || nprobe_max <= 0 || kmax <= 0) return MV_ERR_ARG;
  *out = nullptr;
  return guard(ix->ctx, [&] {
    MV_REQUIRE(ix->trained, MV_ERR_STATE, "index is not trained");
    MV_REQUIRE(kmax <= 4096, MV_ERR_ARG, "k must be at most 4096");
    nprobe_max = std::min(nprobe_max, ix->nlist);
    auto pl = std::make_unique<mv_ivfpq_plan>();
    pl->ix = ix;
    pl->max_nq = max_nq;
    pl->nprobe_max = nprobe_max;
    pl->kmax = kmax;
    if (params) pl->params = *params;
    pl->params.form = MV_FORM_FAST;
    // the tuner may change it
    const int nc = std::min(ix->nlist, nprobe_max + std::max(8, nprobe_max / 4));
    pl->cfg.coarse_matrix = pl->params.coarse_path == 2 ||
                            (pl->params.coarse_path == 0 && !(nc <= 32 && umma_kpad(ix->d) <= 256));
    MV_CHECK_CUDA(cudaStreamCreateWithFlags(&pl->stream, cudaStreamNonBlocking));
    pl->x.ensure(sizeof(float) * max_nq * ix->d);
    pl->nprobe_q.ensure(sizeof(int32_t) * max_nq);
    pl->k_q.ensure(sizeof(int32_t) * max_nq);
    pl->order.ensure(sizeof(int32_t) * max_nq);
    pl->out_d.ensure(sizeof(float) * max_nq * kmax);
    pl->out_l.ensure(sizeof(int64_t) * max_nq * kmax);
    pl->counter.ensure(sizeof(int));
    *out = pl.release();
  });
}

int32_t mv_ivfpq_plan_destroy(mv_ivfpq_plan* pl) {
  if (!pl) return MV_ERR_ARG;
  return guard(pl->ix->ctx, [&] {
    cudaStreamSynchronize(pl->stream);
    delete pl;
  });
}

int32_t mv_ivfpq_plan_buffers(mv_ivfpq_plan* pl, float** d_x, int32_t** d_nprobe, int32_t** d_k,
                              int32_t** d_order, float** d_distances, int64_t** d_labels) {
  if (!pl) return MV_ERR_ARG;
  if (d_x) *d_x = pl->x.as<float>();
  if (d_nprobe) *d_nprobe = pl->nprobe_q.as<int32_t>();
  if (d_k) *d_k = pl->k_q.as<int32_t>();
  if (d_order) *d_order = pl->order.as<int32_t>();
  if (d_distances) *d_distances = pl->out_d.as<float>();
  if (d_labels) *d_labels = pl->out_l.as<int64_t>();
  return MV_OK;
}

int32_t mv_ivfpq_plan_set_queries(mv_ivfpq_plan* pl, const float* x, int64_t nq,
                                  const int32_t* nprobe, const int32_t* k) {
  if (!pl || nq < 0) return MV_ERR_ARG;
  return guard(pl->ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(pl->mu);
    plan_set_queries(pl, x, nq, nprobe, k, pl->stream);
  });
}

int32_t mv_ivfpq_plan_tune(mv_ivfpq_plan* pl, int64_t nq, int32_t* config, float* best_ms) {
  if (!pl || nq <= 0) return MV_ERR_ARG;
  return guard(pl->ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(pl->mu);
    MV_REQUIRE(nq <= pl->max_nq, MV_ERR_ARG, "batch larger than the plan");
    const float ms = plan_tune(pl, nq, pl->stream);
    if (best_ms) *best_ms = ms;
    if (config) {
      config[0] = pl->cfg.coarse_matrix ? 1 : 0;
      config[1] = pl->cfg.scan_threads;
      config[2] = pl->cfg.scan_ctas_per_sm;
    }
    check_kernel_errors(pl->ix->ctx, pl->stream);
  });
}

int32_t mv_ivfpq_plan_run(mv_ivfpq_plan* pl, int64_t nq, int32_t use_graph, void* stream) {
  if (!pl || nq < 0) return MV_ERR_ARG;
  return guard(pl->ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(pl->mu);
    MV_REQUIRE(nq <= pl->max_nq, MV_ERR_ARG, "batch larger than the plan");
    if (nq == 0) return;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : pl->stream;
    plan_run(pl, nq, s, use_graph != 0);
    if (!stream) check_kernel_errors(pl->ix->ctx, s);
  });
}

int32_t mv_ivfpq_plan_results(mv_ivfpq_plan* pl, int64_t nq, float* distances, int64_t* labels) {
  if (!pl || nq < 0 || (nq > 0 && (!distances || !labels))) return MV_ERR_ARG;
  return guard(pl->ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(pl->mu);
    MV_REQUIRE(nq <= pl->max_nq, MV_ERR_ARG, "batch larger than the plan");
    MV_CHECK_CUDA(cudaDeviceSynchronize());  // results of runs on any stream
    d2h(distances, pl->out_d.p, sizeof(float) * nq * pl->kmax, pl->stream);
    d2h(labels, pl->out_l.p, sizeof(int64_t) * nq * pl->kmax, pl->stream);
    sync(pl->stream);
  });
}

int32_t mv_ivfpq_search_batch(mv_ivfpq* ix, const float* x, int64_t nq, const int32_t* nprobe,
                              const int32_t* k, int32_t kmax, const mv_search_params* params,
                              float* distances, int64_t* labels) {
  if (!ix || nq < 0 || kmax <= 0 || (nq > 0 && (!x || !nprobe || !k || !distances || !labels)))
    return MV_ERR_ARG;
  if (nq == 0) return MV_OK;
  int32_t npmax = 1;
  for (int64_t i = 0; i < nq; ++i) npmax = std::max(npmax, nprobe[i]);
  mv_ivfpq_plan* pl = nullptr;
  int32_t st = mv_ivfpq_plan_create(ix, nq, npmax, kmax, params, &pl);
  if (st != MV_OK) return st;
  st = guard(ix->ctx, [&] {
    plan_set_queries(pl, x, nq, nprobe, k, pl->stream);
    plan_run(pl, nq, pl->stream, false);
    d2h(distances, pl->out_d.p, sizeof(float) * nq * kmax, pl->stream);
    d2h(labels, pl->out_l.p, sizeof(int64_t) * nq * kmax, pl->stream);
    check_kernel_errors(ix->ctx, pl->stream);
  });
  mv_ivfpq_plan_destroy(pl);
  return st;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// IVF-Flat (index/index_ivf_flat.mojo)
// ---------------------------------------------------------------------------
namespace mv {

// index_ivf_flat.mojo:91-135: nearest centroid (quantizer search k = 1),
// rows appended to their list in input order.
void ivfflat_add(mv_ivfflat* ix, const float* x, const int64_t* ids, int64_t n) {
  if (!ix->trained || n == 0) return;  // :103-105
  std::vector<uint32_t> ids32(n);
  for (int64_t i = 0; i < n; ++i) {
    MV_REQUIRE(ids[i] >= 0 && ids[i] <= 0xfffffffell, MV_ERR_ARG,
               "ids must be in [0, 2^32 - 2] for the GPU index");
    ids32[i] = (uint32_t)ids[i];
  }
  SlotLease lease(ix->ctx);
  cudaStream_t s = lease.stream();
  const int d = ix->d, nlist = ix->nlist;
  DevBuf new_rows, assign_d;
  new_rows.ensure((size_t)n * d * 4 + 16);
  assign_d.ensure((size_t)n * 4 + 16);
  h2d(new_rows.p, x, sizeof(float) * n * d, s);
  {
    StageTimer t(ix->ctx, MV_STAGE_COARSE, s);  // :115-118 quantizer.search(x, 1)
    assign_nearest(new_rows.as<float>(), n, d, ix->centroids.as<float>(), nlist, ix->metric, 2,
                   assign_d.as<int32_t>(), nullptr, s);
  }
  const int64_t old_total = ix->h_off[nlist];
  AppendLayout L;  // skipped rows (:126) are parked past the end
  append_layout(ix->ctx, assign_d.as<int32_t>(), n, nlist, ix->d_off.as<int64_t>(), old_total, L, s);
  const int64_t cap = L.cap;
  const int64_t* pos = L.pos_d.as<int64_t>();
  DevBuf ids_d, rows_d, ids_new;
  ids_d.ensure(sizeof(uint32_t) * cap + 16);
  rows_d.ensure(sizeof(float) * cap * d + 16);
  ids_new.ensure(sizeof(uint32_t) * n + 16);
  h2d(ids_new.p, ids32.data(), sizeof(uint32_t) * n, s);
  StageTimer t(ix->ctx, MV_STAGE_APPEND, s);
  if (old_total) {
    scatter_rows(ix->d_ids.p, old_total, 4, pos, ids_d.p, s);
    scatter_rows(ix->d_rows.p, old_total, 4 * d, pos, rows_d.p, s);
  }
  scatter_rows(ids_new.p, n, 4, pos + old_total, ids_d.p, s);
  scatter_rows(new_rows.p, n, 4 * d, pos + old_total, rows_d.p, s);
  sync(s);
  DevBuf& off_d = L.off_d;
  std::vector<int64_t>& new_off = L.new_off;
  std::swap(ix->d_off.p, off_d.p);
  std::swap(ix->d_off.bytes, off_d.bytes);
  std::swap(ix->d_ids.p, ids_d.p);
  std::swap(ix->d_ids.bytes, ids_d.bytes);
  std::swap(ix->d_rows.p, rows_d.p);
  std::swap(ix->d_rows.bytes, rows_d.bytes);
  ix->h_off = new_off;
  ix->ntotal += n;  // :135
}

// Search: plain = the reference's coarse step (exact FP32, canonical
// top-nprobe) then the exact scan; fast = BF16 coarse (fused top-k GEMM or
// distance matrix) with an exact FP32 recheck, then the same exact scan.
void ivfflat_search(mv_ivfflat* ix, const float* d_x, int64_t nq, int k, int nprobe,
                    const mv_search_params* p, float* d_out, int64_t* d_lab, DevBuf& ws,
                    cudaStream_t s) {
  if (nq == 0) return;
  if (!ix->trained || ix->ntotal == 0) {  // :176-180
    launch_fill(d_out, d_lab, nq * k, 1e38f, s);
    return;
  }
  MV_REQUIRE(nprobe <= 8192, MV_ERR_UNSUPPORTED, "nprobe above 8192 is not supported on the GPU");
  const bool fast = p && p->form == MV_FORM_FAST && umma_kpad(ix->d) <= UMMA_TOPK_MAX_K;
  const int kp = umma_kpad(ix->d);
  const int nc = std::min(ix->nlist, nprobe + std::max(8, nprobe / 4));
  const int cpath = p ? p->coarse_path : 0;
  MV_REQUIRE(cpath >= 0 && cpath <= 3, MV_ERR_ARG, "coarse_path must be 0, 1, 2 or 3");
  // As in the fast IVF-PQ search: two-pass GEMM + lists where it applies
  // (automatic, or coarse_path 3), the heap epilogue on request, else the
  // distance matrix.
  const bool twopass = fast && nc <= 32 && kp <= 256 && (cpath == 0 || cpath == 3);
  const bool fused = fast && !twopass && nc <= 64 && cpath == 1;
  const bool cert_coarse = !fast && umma_kpad(ix->d) <= UMMA_TOPK_MAX_K &&
                           std::min(ix->nlist, nprobe + std::max(16, nprobe / 2)) < ix->nlist &&
                           nprobe + std::max(16, nprobe / 2) <= UMMA_TOPK_MAX;
  if (fast || cert_coarse) {
    std::lock_guard<std::mutex> lk(ix->fast_mu);
    if (!ix->fast_ready) {
      ix->d_cent_bf16.ensure((size_t)ix->nlist * kp * 2);
      ix->d_cnorm.ensure((size_t)ix->nlist * 4);
      ix->d_ccert.ensure(2 * sizeof(float));
      launch_to_bf16(ix->centroids.as<float>(), ix->nlist, ix->d,
                     ix->d_cent_bf16.as<__nv_bfloat16>(), ix->d_cnorm.as<float>(), s);
      launch_cert_bounds(ix->d_cnorm.as<float>(), ix->centroids.as<float>(), ix->nlist, ix->d,
                         ix->d_ccert.as<float>(), s);
      sync(s);
      ix->fast_ready = true;
    }
  }
  int64_t qb = std::max<int64_t>(64, (int64_t)(1536ll * 1024 * 1024 / ((int64_t)ix->nlist * 4)));
  qb = std::min<int64_t>({qb, nq, 65535ll * 64});
  const int nseg = fused ? umma_topk_nseg(qb, ix->nlist, ix->d, nc, ix->ctx->num_sms)
                 : twopass ? coarse_topk2_nseg(qb, ix->nlist, ix->d, nc, ix->ctx->num_sms) : 1;
  const int ncand = nseg * (fused ? umma_topk_groups(ix->d, nc) : 1) * next_pow2(nc);
  const int lcap = twopass ? coarse_topk2_cap(nc) : 0;
  const bool list_major = ivfflat_lm_supported(qb, ix->d, nprobe, k);
  const size_t lm_bytes = list_major ? ivfflat_lm_scratch_bytes(qb, nprobe, ix->nlist, k) : 0;
  ws.ensure(ws_bytes((size_t)qb * ix->nlist, 4) + ws_bytes((size_t)qb * nprobe, 8) +
            ws_bytes((size_t)qb * nprobe, 4) * 2 + ws_bytes((size_t)qb * kp, 2) +
            ws_bytes((size_t)qb * ncand, 8) + ws_bytes((size_t)qb, 8) +
            ws_bytes((size_t)qb * nseg * lcap, 8) + ws_bytes((size_t)qb * nseg, 4) +
            ws_bytes((size_t)qb, 4) + ws_bytes(lm_bytes, 1));
  Arena ar(ws);
  float* dmat = ar.take<float>((size_t)qb * ix->nlist);
  uint64_t* ckeys = ar.take<uint64_t>((size_t)qb * nprobe);
  int32_t* probes = ar.take<int32_t>((size_t)qb * nprobe);
  float* term = ar.take<float>((size_t)qb * nprobe);
  __nv_bfloat16* xq = ar.take<__nv_bfloat16>((size_t)qb * kp);
  uint64_t* fkeys = ar.take<uint64_t>((size_t)qb * ncand);
  uint64_t* gthr = ar.take<uint64_t>((size_t)qb);
  uint64_t* clists = ar.take<uint64_t>((size_t)qb * nseg * lcap);
  int* ccounts = ar.take<int>((size_t)qb * nseg);
  uint32_t* cthr = ar.take<uint32_t>((size_t)qb);
  unsigned char* lm_scratch = list_major ? ar.take<unsigned char>(lm_bytes) : nullptr;
  const int kind = ix->metric == MV_METRIC_L2 ? KIND_L2_SIMD8 : KIND_IP_SIMD8;
  for (int64_t q0 = 0; q0 < nq; q0 += qb) {
    const int64_t nb = std::min(qb, nq - q0);
    const float* xb = d_x + q0 * ix->d;
    bool certified = false;
    if (cert_coarse) {
      StageTimer t(ix->ctx, MV_STAGE_COARSE, s);
      certified = coarse_topp_certified(ix->ctx, xb, nb, ix->d, ix->centroids.as<float>(),
                                        ix->d_cent_bf16.as<__nv_bfloat16>(), ix->d_cnorm.as<float>(),
                                        ix->d_ccert.as<float>(), ix->nlist, ix->metric, nprobe,
                                        probes, s);
    }
    if (!certified) {
      StageTimer t(ix->ctx, MV_STAGE_COARSE, s);
      if (!fast) {
        launch_exact_matrix(kind, xb, nb, ix->d, ix->centroids.as<float>(), ix->nlist, ix->d,
                            ix->d, dmat, ix->nlist, s);
      } else {
        launch_to_bf16(xb, nb, ix->d, xq, nullptr, s);
        if (twopass)
          launch_coarse_topk2(xq, nb, ix->d_cent_bf16.as<__nv_bfloat16>(), ix->nlist, ix->d,
                              ix->metric, ix->d_cnorm.as<float>(), nc, nseg, clists, ccounts,
                              cthr, ix->ctx->d_err.as<int>(), s);
        else if (fused)
          launch_umma_topk(xq, nb, ix->d_cent_bf16.as<__nv_bfloat16>(), ix->nlist, ix->d,
                           ix->metric, nullptr, ix->d_cnorm.as<float>(), nc, nseg, nullptr,
                           ncand > next_pow2(nc) ? gthr : nullptr, fkeys, ix->ctx->d_err.as<int>(),
                           s);
        else if (umma_kpad(ix->d) > 256)  // the matrix GEMM keeps K resident: exact past d = 256
          launch_exact_matrix(kind, xb, nb, ix->d, ix->centroids.as<float>(), ix->nlist, ix->d,
                              ix->d, dmat, ix->nlist, s);
        else
          launch_umma_dist(EPI_MATRIX, xq, nb, ix->d_cent_bf16.as<__nv_bfloat16>(), ix->nlist,
                           ix->d, ix->metric, nullptr, ix->d_cnorm.as<float>(), dmat, ix->nlist,
                           nullptr, ix->ctx->d_err.as<int>(), ix->ctx->num_sms, s);
      }
    }
    if (!certified) {
      StageTimer t(ix->ctx, MV_STAGE_SELECT, s);
      if (!fast) {  // :185-194 coarse quantizer search with k = nprobe
        launch_select_rows(dmat, nb, ix->nlist, ix->nlist, 0, nprobe, nullptr, ckeys, nullptr, s);
        launch_keys_to_ids(ckeys, nb * nprobe, probes, s);
      } else if (twopass) {
        launch_coarse_lists(clists, ccounts, nseg, lcap, nb, ix->nlist, xb, ix->d,
                            ix->centroids.as<float>(), ix->metric, nc, nprobe, probes, term,
                            ix->ctx->d_err.as<int>(), s);
      } else if (fused) {
        launch_coarse_from_keys(fkeys, nb, ncand, xb, ix->d, ix->centroids.as<float>(), ix->nlist,
                                ix->metric, nc, nprobe, probes, term, ix->ctx->d_err.as<int>(), s);
      } else if (nc <= 64) {
        launch_coarse_rows(dmat, nb, ix->nlist, xb, ix->d, ix->centroids.as<float>(), ix->metric,
                           nc, nprobe, probes, term, ix->ctx->d_err.as<int>(), s);
      } else {
        launch_coarse_fast(dmat, nb, ix->nlist, xb, ix->d, ix->centroids.as<float>(), ix->metric,
                           nc, nprobe, probes, term, ix->ctx->d_err.as<int>(), s);
      }
    }
    StageTimer t(ix->ctx, MV_STAGE_SCAN, s);
    if (list_major)
      launch_ivfflat_scan_lm(xb, nb, ix->d, ix->metric, probes, nprobe, ix->nlist,
                             ix->d_off.as<int64_t>(), ix->d_rows.as<float>(),
                             ix->d_ids.as<uint32_t>(), k, d_out + q0 * k, d_lab + q0 * k,
                             lm_scratch, s);
    else
      launch_ivfflat_scan(xb, nb, ix->d, ix->metric, probes, nprobe, ix->nlist,
                          ix->d_off.as<int64_t>(), ix->d_rows.as<float>(), ix->d_ids.as<uint32_t>(),
                          k, d_out + q0 * k, d_lab + q0 * k, s);
  }
}

}  // namespace mv

extern "C" {

int32_t mv_ivfflat_create(mv_ctx* ctx, int32_t d, int32_t nlist, int32_t metric, mv_ivfflat** out) {
  if (!ctx || !out) return MV_ERR_ARG;
  *out = nullptr;
  return guard(ctx, [&] {
    MV_REQUIRE(d > 0 && d <= 65536, MV_ERR_ARG, "dimension must be between 1 and 65536.");
    MV_REQUIRE(nlist > 0 && nlist <= 1000000, MV_ERR_ARG, "IVF nlist must be between 1 and 1000000.");
    MV_REQUIRE(metric == MV_METRIC_L2 || metric == MV_METRIC_IP, MV_ERR_ARG, "unknown metric");
    auto ix = std::make_unique<mv_ivfflat>();
    ix->ctx = ctx;
    ix->d = d;
    ix->nlist = nlist;
    ix->metric = metric;
    ix->centroids.ensure(sizeof(float) * nlist * d);
    ix->h_off.assign(nlist + 1, 0);
    ix->d_off.ensure(sizeof(int64_t) * (nlist + 1));
    MV_CHECK_CUDA(cudaMemset(ix->d_off.p, 0, sizeof(int64_t) * (nlist + 1)));
    *out = ix.release();
  });
}

int32_t mv_ivfflat_destroy(mv_ivfflat* ix) {
  if (!ix) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    cudaDeviceSynchronize();
    delete ix;
  });
}

int32_t mv_ivfflat_set_nprobe(mv_ivfflat* ix, int32_t nprobe) {
  if (!ix || nprobe < 1) return MV_ERR_ARG;
  ix->nprobe = nprobe;
  return MV_OK;
}

int64_t mv_ivfflat_ntotal(mv_ivfflat* ix) { return ix ? ix->ntotal : -1; }

int32_t mv_ivfflat_train(mv_ivfflat* ix, const float* x, int64_t n, int32_t niter,
                         const mv_search_params* params) {
  if (!ix || (!x && n > 0) || niter < 0) return MV_ERR_ARG;
  const int form = params ? params->form : MV_FORM_PLAIN;
  return guard(ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(ix->mu);
    if (ix->trained) return;  // :71
    MV_REQUIRE(n > 0, MV_ERR_ARG, "training needs at least one vector");
    SlotLease lease(ix->ctx);
    cudaStream_t s = lease.stream();
    DevBuf dx, assign, scratch;
    dx.ensure(sizeof(float) * n * ix->d);
    assign.ensure(sizeof(int32_t) * n);
    h2d(dx.p, x, sizeof(float) * n * ix->d, s);
    // :73-77 KMeans(d, nlist, 15)
    if (form == MV_FORM_FAST && umma_kpad(ix->d) <= UMMA_TOPK_MAX_K)
      kmeans_train_fast(dx.as<float>(), n, ix->d, ix->nlist, niter, ix->centroids.as<float>(),
                        assign.as<int32_t>(), scratch, ix->ctx, s, nullptr);
    else
      kmeans_train_device(dx.as<float>(), n, ix->d, ix->nlist, niter, 1, ix->centroids.as<float>(),
                          assign.as<int32_t>(), scratch, s);
    sync(s);
    ix->trained = true;
    ix->fast_ready = false;
  });
}

int32_t mv_ivfflat_get_centroids(mv_ivfflat* ix, float* out) {
  if (!ix || !out) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    MV_CHECK_CUDA(cudaMemcpy(out, ix->centroids.p, sizeof(float) * ix->nlist * ix->d,
                             cudaMemcpyDeviceToHost));
  });
}

int32_t mv_ivfflat_add_with_ids(mv_ivfflat* ix, const float* x, const int64_t* ids, int64_t n) {
  if (!ix || n < 0 || (n > 0 && (!x || !ids))) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(ix->mu);
    ivfflat_add(ix, x, ids, n);
  });
}

int32_t mv_ivfflat_add(mv_ivfflat* ix, const float* x, int64_t n) {
  if (!ix || n < 0 || (n > 0 && !x)) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    std::lock_guard<std::mutex> lk(ix->mu);
    std::vector<int64_t> ids(n);
    for (int64_t i = 0; i < n; ++i) ids[i] = ix->ntotal + i;  // :86-89
    ivfflat_add(ix, x, ids.data(), n);
  });
}

int32_t mv_ivfflat_search(mv_ivfflat* ix, const float* x, int64_t nq, int32_t k,
                          const mv_search_params* params, float* distances, int64_t* labels) {
  if (!ix || (nq > 0 && (!x || !distances || !labels))) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    check_search_args(nq, k);
    if (nq == 0) return;
    int nprobe = params && params->nprobe > 0 ? params->nprobe : ix->nprobe;
    nprobe = std::min(nprobe, ix->nlist);  // :182-183
    SlotLease lease(ix->ctx);
    cudaStream_t s = lease.stream();
    DevBuf& io = lease.slot->io;
    io.ensure(ws_bytes((size_t)nq * ix->d, 4) + ws_bytes((size_t)nq * k, 4) +
              ws_bytes((size_t)nq * k, 8));
    Arena ar(io);
    float* dx = ar.take<float>((size_t)nq * ix->d);
    float* dd = ar.take<float>((size_t)nq * k);
    int64_t* dl = ar.take<int64_t>((size_t)nq * k);
    h2d(dx, x, sizeof(float) * nq * ix->d, s);
    ivfflat_search(ix, dx, nq, k, nprobe, params, dd, dl, lease.slot->ws, s);
    d2h(distances, dd, sizeof(float) * nq * k, s);
    d2h(labels, dl, sizeof(int64_t) * nq * k, s);
    check_kernel_errors(ix->ctx, s);
  });
}

int32_t mv_ivfflat_search_device(mv_ivfflat* ix, const float* d_x, int64_t nq, int32_t k,
                                 const mv_search_params* params, float* d_distances,
                                 int64_t* d_labels, void* stream) {
  if (!ix || (nq > 0 && (!d_x || !d_distances || !d_labels))) return MV_ERR_ARG;
  return guard(ix->ctx, [&] {
    check_search_args(nq, k);
    if (nq == 0) return;
    int nprobe = params && params->nprobe > 0 ? params->nprobe : ix->nprobe;
    nprobe = std::min(nprobe, ix->nlist);
    SlotLease lease(ix->ctx);
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : lease.stream();
    lease.use(s);
    ivfflat_search(ix, d_x, nq, k, nprobe, params, d_distances, d_labels, lease.slot->ws, s);
    if (!stream) check_kernel_errors(ix->ctx, s);
  });
}

}  // extern "C"
