// Host-side internals of libmojovec_gpu.so: context, device buffers, the
// per-call stream/workspace pool and the index objects behind the C ABI.
#pragma once

#include <functional>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mojovec_gpu.h"

namespace mv {

// Error carried through the C++ layer and turned into a status code at the
// C boundary.
struct Error : std::runtime_error {
  int32_t code;
  Error(int32_t c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

#define MV_CHECK_CUDA(expr)                                                          \
  do {                                                                               \
    cudaError_t _e = (expr);                                                         \
    if (_e != cudaSuccess)                                                           \
      throw ::mv::Error(MV_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

#define MV_REQUIRE(cond, code, msg)                  \
  do {                                               \
    if (!(cond)) throw ::mv::Error((code), (msg));   \
  } while (0)

// Owning device allocation (grow-only).
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  void ensure(size_t n) {
    if (n <= bytes) return;
    release();
    if (n == 0) return;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      p = nullptr;
      throw Error(MV_ERR_OOM, std::string("cudaMalloc(") + std::to_string(n) + "): " + cudaGetErrorString(e));
    }
    bytes = n;
  }
  template <typename T>
  T* as() const { return static_cast<T*>(p); }
};

// Bump allocator over a workspace buffer for one call.
struct Arena {
  char* base;
  size_t cap, off = 0;
  Arena(DevBuf& buf) : base(buf.as<char>()), cap(buf.bytes) {}
  template <typename T>
  T* take(size_t count) {
    size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
    MV_REQUIRE(off + bytes <= cap, MV_ERR_INTERNAL, "workspace overflow");
    T* r = reinterpret_cast<T*>(base + off);
    off += bytes;
    return r;
  }
};
inline size_t ws_bytes(size_t count, size_t elem) { return (count * elem + 255) & ~size_t(255); }

// Raises a kernel's dynamic shared-memory limit to at least `bytes`. The
// limit only ever grows (a per-kernel high-water mark), so a concurrent
// launch that needs more is never undercut by one that needs less. Needed
// whenever static + dynamic shared memory exceeds 48 KB.
void raise_smem_limit(const void* kernel, size_t bytes);
// Runs f with ctx as the calling thread's current context (its device set,
// its launch counter counting) and turns exceptions into status codes and
// the thread's last error message, as every entry point does.
int32_t guarded(mv_ctx* ctx, const std::function<void()>& f);
// The pipeline-wait limit (cycles) of the calling thread's current context
// (the default when there is none), copied into each tensor-core launch.
long long current_wait_limit();
template <typename K>
inline void smem_limit(K kernel, size_t bytes) {
  raise_smem_limit(reinterpret_cast<const void*>(kernel), bytes);
}

// One per concurrent call: its own stream and scratch, so concurrent
// read-only searches (the reference releases the GIL around search,
// python/mojovec_python.mojo:1074) never share mutable state.
struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;  // recorded on release; the slot is reused only after it
  DevBuf ws;                   // internal scratch
  DevBuf io;                   // device copies of host inputs/outputs
};

}  // namespace mv

struct mv_ctx {
  int device = 0;
  int num_sms = 0;
  size_t smem_optin = 0;
  std::mutex mu;
  std::vector<mv::Slot*> free_slots;
  std::vector<mv::Slot*> all_slots;
  std::atomic<int64_t> launches{0};
  cudaStream_t main_stream = nullptr;
  mv::DevBuf d_err;  // int: set by kernels whose bounded waits gave up
  // cycles a tensor-core kernel's pipeline wait may take before it gives up
  // (mv_ctx_set_wait_limit); 0 = give up at once unless already complete
  std::atomic<long long> wait_limit{4000000000ll};
  // certified selections (mv_ctx_certify_stats): nearest-centroid rows and
  // plain Flat queries, and how many of each the bound left to the exact scan
  std::atomic<int64_t> assign_rows{0}, assign_fallback{0}, flat_queries{0}, flat_fallback{0};
  // stage profiling (mv_ctx_profile)
  std::atomic<bool> profile{false};
  std::mutex prof_mu;
  struct StageRec {
    int stage;
    cudaEvent_t a, b;
  };
  std::vector<StageRec> prof_pending;
  double stage_ms[MV_STAGE_COUNT] = {};
  int64_t stage_n[MV_STAGE_COUNT] = {};

  mv::Slot* acquire();
  void release(mv::Slot* s, cudaStream_t used);
  void set_device() const;
};

namespace mv {

// RAII stage bracket: records a CUDA event pair on `s` when profiling is on.
struct StageTimer {
  mv_ctx* ctx;
  int stage;
  cudaStream_t s;
  cudaEvent_t a = nullptr;
  StageTimer(mv_ctx* c, int st, cudaStream_t stream) : ctx(c), stage(st), s(stream) {
    if (ctx && ctx->profile.load()) {
      cudaEventCreate(&a);
      cudaEventRecord(a, s);
    }
  }
  ~StageTimer() {
    if (!a) return;
    cudaEvent_t b;
    cudaEventCreate(&b);
    cudaEventRecord(b, s);
    std::lock_guard<std::mutex> lk(ctx->prof_mu);
    ctx->prof_pending.push_back({stage, a, b});
  }
};

// RAII: acquire a pool slot for the duration of one C-ABI call.
// The lease records the stream the call ran on; release() records an event
// there so a later call reuses the slot's buffers only after this call's
// kernels finished (calls may return before their stream drains).
struct SlotLease {
  mv_ctx* ctx;
  Slot* slot;
  cudaStream_t used;
  explicit SlotLease(mv_ctx* c) : ctx(c), slot(c->acquire()), used(slot->stream) {}
  ~SlotLease() { ctx->release(slot, used); }
  cudaStream_t stream() const { return slot->stream; }
  void use(cudaStream_t s) { used = s; }
};

// Per-query parameters and launch shapes of a batched fast IVF-PQ search.
struct FastBatch {
  const int32_t* nprobe_q = nullptr;  // device, per query
  const int32_t* k_q = nullptr;       // device, per query
  const int32_t* order = nullptr;     // device, scan order (a permutation)
  int* counter = nullptr;             // device, persistent scan work counter
  int scan_threads = 256;             // 128, 256 or 512
  int scan_ctas_per_sm = 4;           // persistent grid size; 0 = one CTA per query
  bool coarse_matrix = false;         // distance matrix + select even where the fused GEMM fits
};

}  // namespace mv

struct mv_ivfpq {
  mv_ctx* ctx;
  int d, nlist, M, dsub, metric, nprobe = 1;
  bool trained = false;
  int64_t ntotal = 0;
  std::mutex mu;
  mv::DevBuf centroids;   // nlist x d FP32 (IndexFlat quantizer rows)
  mv::DevBuf pq;          // M x 256 x dsub FP32
  // Inverted lists (storage/inverted_lists.mojo:37) flattened to CSR in
  // list order on the device; entries of a list keep append order.
  std::vector<int64_t> h_off;     // nlist + 1 (host copy of the offsets)
  mv::DevBuf d_off;     // int64 nlist + 1
  mv::DevBuf d_ids;     // uint32 per entry
  mv::DevBuf d_codes;   // M bytes per entry
  mv::DevBuf d_raw;     // FP32 rows per entry (exact rerank in the fast form)
  bool has_raw = true;  // false when the lists came without rows (snapshot, set_lists)
  // Collection metadata carried through snapshots (api/collection_ivfpq.mojo).
  std::vector<int64_t> user_ids;
  std::string coll_name, coll_metric;
  // Fast-form state (built lazily from the above).
  std::mutex fast_mu;
  bool fast_ready = false;
  bool coarse_ready = false;  // d_cent_bf16, d_cnorm, d_ccert (centroid-only state)
  mv::DevBuf d_ccert;       // 2 floats: bound on ||bf16(c)||^2, max ||c - bf16(c)||
  mv::DevBuf d_vec_term;    // FP32 per vector: ||y||^2 + 2<c, y> (y = PQ reconstruction)
  mv::DevBuf d_raw8;        // 8-bit rows per entry, d8 bytes (certified rerank prescreen)
  mv::DevBuf d_rmeta;       // float2 per entry: bounds on ||y - y8|| and ||y8||
  mv::DevBuf d_dim8;        // float2 per dimension: offset a_j, power-of-two step s_j
  mv::DevBuf d_dimord;      // 2 x d ordered words: per-dimension minimum and maximum
  mv::DevBuf d_pq16;        // FP16 codebook * pq16_scale (fast-form tables; dsub 4 or 8)
  float pq16_inv = 0.0f;    // 1 / scale; 0 = no FP16 codebook
  mv::DevBuf d_pq_cn;       // FP32 per subspace: bound on its largest codeword norm
  bool has_pq_cn = false;
  mv::DevBuf d_cnorm;       // FP32 per centroid ||c||^2
  mv::DevBuf d_cent_bf16;   // nlist x d BF16
  // longest[i]: total rows of the i longest lists (i = 0..nlist): bounds
  // the candidate count of a query probing i lists
  std::vector<int64_t> longest;
};

struct mv_ivfflat {
  mv_ctx* ctx;
  int d, nlist, metric, nprobe = 1;
  bool trained = false;
  int64_t ntotal = 0;
  std::mutex mu;
  mv::DevBuf centroids;           // nlist x d FP32 (quantizer rows)
  std::vector<int64_t> h_off;     // nlist + 1
  mv::DevBuf d_off;               // int64 nlist + 1
  mv::DevBuf d_ids;               // uint32 per entry
  mv::DevBuf d_rows;              // FP32 rows per entry, in list order
  std::mutex fast_mu;
  bool fast_ready = false;
  mv::DevBuf d_cent_bf16, d_cnorm;  // fast coarse step
  mv::DevBuf d_ccert;               // 2 floats: coarse certificate bounds
};

struct mv_flat {
  mv_ctx* ctx;
  int d, metric;
  int64_t ntotal = 0, capacity = 0;
  std::mutex mu;
  mv::DevBuf rows;       // capacity x d FP32
  mv::DevBuf rows_bf16;  // ntotal x kpad BF16 (fast form, built lazily)
  mv::DevBuf norms;      // FP32 ||x||^2 per rounded row (fast form)
  mv::DevBuf cert;       // 2 floats: bound on ||bf16(y)||^2, max ||y - bf16(y)|| (fast form)
  mv::DevBuf rows_e4m3;  // ntotal x umma_kpad8(d) E4M3 rows (fast form with flat_e4m3)
  mv::DevBuf scales_e4m3, norms_e4m3;  // per row: scale, norm of the dequantized row
  bool e4m3_ready = false;
  std::mutex fast_mu;
  bool fast_ready = false;
  int64_t overflow_rows = 0;  // fast-form queries recomputed exactly (shortlist overflow)
};

struct mv_sq8 {
  mv_ctx* ctx;
  int d, dpad, metric;
  int64_t ntotal = 0, capacity = 0;
  float gmin, gmax, scale = 1.0f;
  std::mutex mu;
  mv::DevBuf f32;    // capacity x d
  mv::DevBuf codes;  // capacity x dpad (zero padded)
  mv::DevBuf norms;  // capacity uint32
  // Tensor-core scan state (built lazily): codes as BF16 rows, norms as FP32.
  std::mutex fast_mu;
  bool fast_ready = false;
  mv::DevBuf codes_bf16;
  mv::DevBuf fnorms;
  int64_t fallback_rows = 0;  // queries rescanned because of a possible tie
};
