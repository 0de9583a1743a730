// Row-wise k-selection over distance matrices and key decoding.
//
// Replaces the per-query heaps of IndexFlat._search_impl
// (index/index_flat.mojo:284-316) for the coarse top-nprobe step and the
// plain Flat scan. One CTA owns one row (query): it streams the row's
// distances with coalesced loads, keeps the canonical k smallest
// (distance, id) keys with BlockTopK and can seed from the previous chunk's
// keys, so a scan split into column chunks gives the same answer as one
// pass.
#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"

namespace mv {
namespace {

constexpr int SEL_THREADS = 256;
constexpr int SEL_BUF = 512;

__global__ void __launch_bounds__(SEL_THREADS)
    k_select_rows(const float* __restrict__ D, int64_t ldd, int64_t ncols, int64_t col_base, int k,
                  const uint64_t* __restrict__ prev, uint64_t* __restrict__ out,
                  const uint8_t* __restrict__ filter) {
  extern __shared__ uint64_t skeys[];
  __shared__ int cnt;
  __shared__ uint64_t thr;
  const int64_t r = blockIdx.x;
  BlockTopK sel;
  sel.init(skeys, &cnt, &thr, k, SEL_BUF);
  if (prev) sel.seed(prev + r * k);
  const float* row = D + r * ldd;
  for (int64_t c0 = 0; c0 < ncols; c0 += SEL_THREADS) {
    int64_t c = c0 + threadIdx.x;
    if (c < ncols) {
      int64_t gid = col_base + c;
      if (!filter || filter[gid] == 0) sel.push(make_key(row[c], (uint32_t)gid));
    }
    sel.end_round();
  }
  sel.finish();
  for (int i = threadIdx.x; i < k; i += SEL_THREADS) out[r * k + i] = skeys[i];
}

__global__ void k_keys_to_results(const uint64_t* __restrict__ keys, int64_t total, float fill_d,
                                  int negate, float* __restrict__ out_d,
                                  int64_t* __restrict__ out_l) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  uint64_t key = keys[i];
  if (key == KEY_NONE) {
    out_d[i] = fill_d;
    out_l[i] = -1;
  } else {
    float dd = key_dist(key);
    out_d[i] = negate ? -dd : dd;
    out_l[i] = (int64_t)key_id(key);
  }
}

__global__ void k_keys_to_ids(const uint64_t* __restrict__ keys, int64_t n, int32_t* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t key = keys[i];
  out[i] = (key == KEY_NONE) ? -1 : (int32_t)key_id(key);
}

}  // namespace

void launch_select_rows(const float* D, int64_t rows, int64_t ldd, int64_t ncols,
                        int64_t col_base, int k, const uint64_t* prev, uint64_t* out,
                        const uint8_t* filter, cudaStream_t s) {
  if (rows == 0) return;
  MV_REQUIRE(rows <= 0x7fffffff, MV_ERR_UNSUPPORTED, "too many rows");
  size_t smem = (size_t)BlockTopK::smem_keys(k, SEL_BUF) * sizeof(uint64_t);
  MV_REQUIRE(smem <= 200 * 1024, MV_ERR_UNSUPPORTED, "k too large for the select kernel");
  smem_limit(k_select_rows, smem);
  k_select_rows<<<(unsigned)rows, SEL_THREADS, smem, s>>>(D, ldd, ncols, col_base, k, prev, out,
                                                           filter);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_keys_to_results(const uint64_t* keys, int64_t rows, int k, float fill_d, bool negate,
                            float* out_d, int64_t* out_l, cudaStream_t s) {
  int64_t total = rows * k;
  if (total == 0) return;
  k_keys_to_results<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(keys, total, fill_d,
                                                                    negate ? 1 : 0, out_d, out_l);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_keys_to_ids(const uint64_t* keys, int64_t n, int32_t* out, cudaStream_t s) {
  if (n == 0) return;
  k_keys_to_ids<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(keys, n, out);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
