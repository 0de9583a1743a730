// Fast k-means step (clustering/kmeans.mojo:84-220 semantics for the
// assignment rule and the empty-cluster reseed; the sums in FP64).
//
// Assign: the BF16 tensor-core GEMM with the per-row heap epilogue keeps,
// per row, the few centroids with the smallest BF16 distances; k_km_recheck
// recomputes those candidates with the reference's FP32 distance
// (l2_distance_simd[8], or the short4 form for d <= 4) and keeps the
// smallest, the smaller index on equal distances (the reference's strict
// `<` over centroids in index order). Only a centroid that the BF16
// ranking pushed out of the candidates can be missed.
//
// Update: the centroid sums are accumulated in FP64 in a fixed order, so
// the step is deterministic: a stable counting sort groups the rows by
// cluster (per-tile histograms, a column scan over tiles, an exclusive scan
// over clusters, then an in-order placement per tile), and thread (c, j)
// adds x[i][j] over cluster c's rows in row order. centroid = sum * (1 /
// count) in FP64, rounded to FP32; an empty cluster takes row
// (offset + (it + 1) * k + c) % n (kmeans.mojo:211-220).
#include "mv_exact.cuh"
#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"

namespace mv {
namespace {

constexpr int KT = 4096;  // rows per tile of the counting sort

// One warp per row: exact FP32 distances of the candidate centroids.
__global__ void k_km_recheck(const float* __restrict__ x, int64_t n, int d,
                             const float* __restrict__ cent, int k, const uint64_t* __restrict__ cand,
                             int ncand, int32_t* __restrict__ assign, float* __restrict__ mind) {
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float* xr = x + row * d;
  // each lane evaluates candidates lane, lane + 32, ... (the whole distance)
  float best = __int_as_float(0x7f800000);
  int bi = 0x7fffffff;
  for (int c = lane; c < ncand; c += 32) {
    const uint64_t key = cand[row * ncand + c];
    if (key == KEY_NONE) continue;
    const uint32_t ci = key_id(key);
    if (ci >= (uint32_t)k) continue;
    const float dd = d <= 4 ? l2_short4(xr, cent + (int64_t)ci * d, d)
                            : l2_simd<8>(xr, cent + (int64_t)ci * d, d);
    const float v = fmaxf(dd, 0.0f);
    if (v < best || (v == best && (int)ci < bi)) {
      best = v;
      bi = (int)ci;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ob < best || (ob == best && oi < bi)) {
      best = ob;
      bi = oi;
    }
  }
  if (lane == 0) {
    assign[row] = bi == 0x7fffffff ? 0 : bi;
    mind[row] = bi == 0x7fffffff ? 0.0f : best;
  }
}

// hist[t][c]: rows of tile t assigned to cluster c.
__global__ void k_km_hist(const int32_t* __restrict__ assign, int64_t n, int k,
                          int32_t* __restrict__ hist) {
  extern __shared__ int32_t cnt[];
  const int64_t t = blockIdx.x;
  for (int c = threadIdx.x; c < k; c += blockDim.x) cnt[c] = 0;
  __syncthreads();
  const int64_t r0 = t * KT, r1 = r0 + KT < n ? r0 + KT : n;
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) atomicAdd(&cnt[assign[r]], 1);
  __syncthreads();
  for (int c = threadIdx.x; c < k; c += blockDim.x) hist[t * k + c] = cnt[c];
}

// base[t][c] = rows of cluster c in tiles before t; total[c].
__global__ void k_km_colscan(int32_t* __restrict__ hist, int ntiles, int k,
                             int32_t* __restrict__ total) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  int run = 0;
  for (int t = 0; t < ntiles; ++t) {
    const int h = hist[(int64_t)t * k + c];
    hist[(int64_t)t * k + c] = run;
    run += h;
  }
  total[c] = run;
}

// start[c] = sum of total[c'] over c' < c (one block).
__global__ void k_km_exscan(const int32_t* __restrict__ total, int k, int32_t* __restrict__ start) {
  __shared__ int32_t part[1024];
  const int per = (k + blockDim.x - 1) / blockDim.x;
  const int c0 = threadIdx.x * per;
  int s = 0;
  for (int c = c0; c < min(c0 + per, k); ++c) s += total[c];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      const int v = part[i];
      part[i] = run;
      run += v;
    }
  }
  __syncthreads();
  int run = part[threadIdx.x];
  for (int c = c0; c < min(c0 + per, k); ++c) {
    start[c] = run;
    run += total[c];
  }
}

// One warp per tile places its rows in row order: perm[pos] = row.
__global__ void k_km_place(const int32_t* __restrict__ assign, int64_t n, int k,
                           const int32_t* __restrict__ base, const int32_t* __restrict__ start,
                           int32_t* __restrict__ perm) {
  extern __shared__ int32_t cur[];
  const int64_t t = blockIdx.x;
  const int lane = threadIdx.x;
  for (int c = lane; c < k; c += 32) cur[c] = start[c] + base[t * k + c];
  __syncwarp();
  const int64_t r0 = t * KT, r1 = r0 + KT < n ? r0 + KT : n;
  for (int64_t g = r0; g < r1; g += 32) {
    const int64_t r = g + lane;
    const bool ok = r < r1;
    const int c = ok ? assign[r] : -1 - lane;  // distinct for idle lanes
    const unsigned peers = __match_any_sync(0xffffffffu, c);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    const int leader = __ffs(peers) - 1;
    int pos = 0;
    if (ok) pos = cur[c] + rank;
    __syncwarp();
    if (ok && lane == leader) cur[c] += __popc(peers);
    __syncwarp();
    if (ok) perm[pos] = (int32_t)r;
  }
}

// Thread (c, j): FP64 sum over cluster c's rows in row order -> centroid.
__global__ void k_km_sums(const float* __restrict__ x, int64_t n, int d, int k,
                          const int32_t* __restrict__ perm, const int32_t* __restrict__ start,
                          const int32_t* __restrict__ total, int64_t sample_offset, int it,
                          float* __restrict__ cent) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)k * d) return;
  const int c = (int)(e / d);
  const int j = (int)(e - (int64_t)c * d);
  const int cnt = total[c];
  if (cnt == 0) {  // kmeans.mojo:211-220
    const int64_t src = (sample_offset + (int64_t)(it + 1) * k + c) % n;
    cent[e] = x[src * d + j];
    return;
  }
  const int32_t* rows = perm + start[c];
  double s = 0.0;
  for (int i = 0; i < cnt; ++i) s += (double)x[(int64_t)rows[i] * d + j];
  cent[e] = (float)(s * (1.0 / (double)cnt));
}

// Deterministic FP64 sum of n values: per-block partials (fixed order),
// then one block adds the partials in order.
__global__ void k_km_partial(const float* __restrict__ v, int64_t n, double* __restrict__ part) {
  __shared__ double sm[256];
  const int64_t per = (n + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = (int64_t)blockIdx.x * per, b1 = b0 + per < n ? b0 + per : n;
  double s = 0.0;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) s += (double)v[i];
  sm[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

__global__ void k_km_final(const double* __restrict__ part, int np, double* __restrict__ out) {
  double s = 0.0;
  for (int i = 0; i < np; ++i) s += part[i];
  *out = s;
}

}  // namespace

void launch_km_recheck(const float* x, int64_t n, int d, const float* cent, int k,
                       const uint64_t* cand, int ncand, int32_t* assign, float* mind,
                       cudaStream_t s) {
  if (n == 0) return;
  k_km_recheck<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(x, n, d, cent, k, cand, ncand, assign, mind);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

size_t km_sort_scratch_bytes(int64_t n, int k) {
  const int64_t ntiles = (n + KT - 1) / KT;
  return (size_t)(ntiles * k + 2 * (int64_t)k + n) * sizeof(int32_t) + 4 * 256;
}

void launch_km_update_fp64(const float* x, int64_t n, int d, int k, const int32_t* assign,
                           int64_t sample_offset, int it, float* cent, void* scratch,
                           cudaStream_t s) {
  if (n == 0) return;
  MV_REQUIRE((size_t)k * 4 <= 200 * 1024, MV_ERR_UNSUPPORTED, "fast k-means: k above 51200");
  const int64_t ntiles = (n + KT - 1) / KT;
  int32_t* hist = static_cast<int32_t*>(scratch);
  int32_t* total = hist + ntiles * k;
  int32_t* start = total + k;
  int32_t* perm = start + k;
  const size_t smem = (size_t)k * 4;
  smem_limit(k_km_hist, smem);
  k_km_hist<<<(unsigned)ntiles, 256, smem, s>>>(assign, n, k, hist);
  k_km_colscan<<<(unsigned)((k + 255) / 256), 256, 0, s>>>(hist, (int)ntiles, k, total);
  k_km_exscan<<<1, 1024, 0, s>>>(total, k, start);
  smem_limit(k_km_place, smem);
  k_km_place<<<(unsigned)ntiles, 32, smem, s>>>(assign, n, k, hist, start, perm);
  const int64_t kd = (int64_t)k * d;
  k_km_sums<<<(unsigned)((kd + 255) / 256), 256, 0, s>>>(x, n, d, k, perm, start, total,
                                                          sample_offset, it, cent);
  for (int i = 0; i < 5; ++i) count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_sum_fp64(const float* v, int64_t n, double* part256, double* out, cudaStream_t s) {
  k_km_partial<<<256, 256, 0, s>>>(v, n, part256);
  k_km_final<<<1, 1, 0, s>>>(part256, 256, out);
  count_launch();
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
