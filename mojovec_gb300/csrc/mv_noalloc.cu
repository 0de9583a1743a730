// mv_ivfpq_search_noalloc: the plain IVF-PQ search without any device-memory
// allocation.
//
// Some callers cannot allocate device memory while they search: a serving
// process that hands all GPU memory to its own pool at start-up (where
// cudaMalloc would fail or take memory the pool counts on), and hosts that
// must not let cudaFree's implicit device synchronisation stall other work
// in a latency-critical loop. For them this entry point takes device inputs
// and outputs from the caller and keeps its own scratch (the coarse distance
// matrix, the coarse keys and the probe lists) in one fixed array of
// MV_NOALLOC_SCRATCH_BYTES declared below. Every GPU that loads the library
// holds that array until the process exits.
//
// Set-up: the first call on a device (with that device current) resolves
// the array's device address with cudaGetSymbolAddress and caches it; make
// that first call before any stream capture. Host code never passes the
// array's name to a kernel: in host code it is only a stand-in symbol.
//
// Sharing: every call uses the same array and leaves its contents behind.
// Nothing in it has to start at zero (each region is written before it is
// read). Calls whose work overlaps on the GPU (different streams, or
// different host threads) race on the array; serialise them.
#include <mutex>

#include "mv_internal.h"
#include "mv_kernels.h"

namespace mv {
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[MV_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;

// Device address of g_noalloc_scratch for the current device (resolved once
// per device).
unsigned char* noalloc_scratch() {
  static std::mutex mu;
  static unsigned char* addr[kMaxDevices] = {};
  int dev = 0;
  MV_CHECK_CUDA(cudaGetDevice(&dev));
  MV_REQUIRE(dev >= 0 && dev < kMaxDevices, MV_ERR_UNSUPPORTED, "device index out of range");
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    MV_REQUIRE(e == cudaSuccess && p != nullptr, MV_ERR_CUDA,
               std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e));
    addr[dev] = static_cast<unsigned char*>(p);
  }
  return addr[dev];
}

__global__ void k_fill_noalloc(float* d, int64_t* l, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    d[i] = 1e38f;
    l[i] = -1;
  }
}

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Scratch bytes for a batch of qb queries.
size_t batch_bytes(int64_t qb, int nlist, int nprobe) {
  return align256((size_t)qb * nlist * 4) + align256((size_t)qb * nprobe * 8) +
         align256((size_t)qb * nprobe * 4);
}

}  // namespace
}  // namespace mv

extern "C" int32_t mv_ivfpq_search_noalloc(mv_ivfpq* ix, const float* d_x, int64_t nq, int32_t k,
                                           int32_t nprobe, float* d_distances, int64_t* d_labels,
                                           void* stream) {
  using namespace mv;
  if (!ix) {
    set_last_error("mv_ivfpq_search_noalloc: null index");
    return MV_ERR_ARG;
  }
  return guarded(ix->ctx, [&] {
    MV_REQUIRE(nq >= 0, MV_ERR_ARG, "mv_ivfpq_search_noalloc: negative query count");
    MV_REQUIRE(nq == 0 || (d_x && d_distances && d_labels), MV_ERR_ARG,
               "mv_ivfpq_search_noalloc: null query or result pointer");
    MV_REQUIRE(k >= 1 && k <= 2048, MV_ERR_ARG, "n_results must be between 1 and 2048.");
    MV_REQUIRE(nprobe >= 0, MV_ERR_ARG, "nprobe must be non-negative");
    if (nq == 0) return;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char* scratch = noalloc_scratch();
    if (!ix->trained || ix->ntotal == 0) {  // index/index_ivf_pq.mojo:247-251
      k_fill_noalloc<<<(unsigned)((nq * k + 255) / 256), 256, 0, s>>>(d_distances, d_labels, nq * k);
      count_launch();
      MV_CHECK_CUDA(cudaGetLastError());
      return;
    }
    const int np = std::min(nprobe > 0 ? (int)nprobe : ix->nprobe, ix->nlist);
    MV_REQUIRE(np <= 8192, MV_ERR_UNSUPPORTED, "nprobe above 8192 is not supported on the GPU");
    const size_t one = batch_bytes(1, ix->nlist, np);
    MV_REQUIRE(one <= MV_NOALLOC_SCRATCH_BYTES, MV_ERR_ARG,
               "mv_ivfpq_search_noalloc: one query needs " + std::to_string(one) +
                   " bytes of scratch, above its fixed " +
                   std::to_string((size_t)MV_NOALLOC_SCRATCH_BYTES) + "-byte maximum");
    int64_t qb = std::min<int64_t>(nq, 65535ll * 64);
    while (qb > 1 && batch_bytes(qb, ix->nlist, np) > MV_NOALLOC_SCRATCH_BYTES) qb /= 2;
    unsigned char* p0 = scratch;
    float* dmat = reinterpret_cast<float*>(p0);
    uint64_t* ckeys = reinterpret_cast<uint64_t*>(p0 + align256((size_t)qb * ix->nlist * 4));
    int32_t* probes = reinterpret_cast<int32_t*>(reinterpret_cast<unsigned char*>(ckeys) +
                                                 align256((size_t)qb * np * 8));
    const int kind = ix->metric == MV_METRIC_L2 ? KIND_L2_SIMD8 : KIND_IP_SIMD8;
    for (int64_t q0 = 0; q0 < nq; q0 += qb) {
      const int64_t nb = std::min(qb, nq - q0);
      const float* xq = d_x + q0 * ix->d;
      launch_exact_matrix(kind, xq, nb, ix->d, ix->centroids.as<float>(), ix->nlist, ix->d, ix->d,
                          dmat, ix->nlist, s);
      launch_select_rows(dmat, nb, ix->nlist, ix->nlist, 0, np, nullptr, ckeys, nullptr, s);
      launch_keys_to_ids(ckeys, nb * np, probes, s);
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
      a.nprobe = np;
      a.filter = nullptr;
      a.filter_len = 0;
      a.k = k;
      a.out_d = d_distances + q0 * k;
      a.out_l = d_labels + q0 * k;
      launch_ivfpq_scan_plain(a, s);
    }
  });
}
