// Plain (reference-exact) k-means update step.
//
// KMeans._train (clustering/kmeans.mojo:84-220) splits the n rows into 32
// fixed chunks; each chunk sums its rows into a chunk-local FP32 accumulator
// in row order, the chunk accumulators are then added in chunk order
// 0..31, and each centroid is multiplied by Float32(1.0) / count.
//
// k_kmeans_accumulate keeps that order exactly: CTA (chunk, 32-dim slice)
// walks its chunk's rows in order, lane j adding x[i][slice*32 + j] into
// the accumulator of cluster assign[i]. The accumulator lives in shared
// memory when k x 32 floats fit, otherwise in the global chunk buffer; in
// both cases each (chunk, cluster, dim) sum is built by a single lane in row
// order, so the FP32 result equals the reference's.
#include "mv_exact.cuh"
#include "mv_internal.h"
#include "mv_kernels.h"

namespace mv {
namespace {

constexpr int NUM_CHUNKS = 32;  // kmeans.mojo:84

__global__ void k_gather_rows(const float* __restrict__ x, int d, const int64_t* __restrict__ idx,
                              int64_t count, float* __restrict__ out, int64_t bx, int64_t bo) {
  x += blockIdx.y * bx;
  out += blockIdx.y * bo;
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= count * d) return;
  int64_t r = e / d;
  int j = (int)(e - r * d);
  out[e] = x[idx[r] * d + j];
}

template <bool SMEM>
__global__ void k_kmeans_accumulate(const float* __restrict__ x, int64_t n, int d, int k,
                                    const int32_t* __restrict__ assign,
                                    float* __restrict__ local_sums,
                                    int32_t* __restrict__ local_counts, int64_t bx, int64_t ba,
                                    int64_t bs, int64_t bc) {
  extern __shared__ float acc_s[];
  const int chunk = blockIdx.x;
  const int slice = blockIdx.y;
  x += blockIdx.z * bx;
  assign += blockIdx.z * ba;
  local_sums += blockIdx.z * bs;
  local_counts += blockIdx.z * bc;
  const int lane = threadIdx.x;
  const int j = slice * 32 + lane;
  const bool active = j < d;
  const int64_t chunk_size = (n + NUM_CHUNKS - 1) / NUM_CHUNKS;
  const int64_t start = (int64_t)chunk * chunk_size;
  const int64_t end = min(start + chunk_size, n);
  float* my_sums = local_sums + (int64_t)chunk * k * d;
  int* cnt_s = reinterpret_cast<int*>(acc_s + (SMEM ? (size_t)k * 32 : 0));
  if (SMEM) {
    for (int e = lane; e < k * 32; e += 32) acc_s[e] = 0.0f;
  } else if (active) {
    for (int c = 0; c < k; ++c) my_sums[(int64_t)c * d + j] = 0.0f;
  }
  const bool do_counts = (slice == 0);
  if (do_counts)
    for (int c = lane; c < k; c += 32) cnt_s[c] = 0;
  __syncwarp();
  // Loads for 8 rows are issued together; the adds are applied strictly in
  // row order.
  constexpr int U = 8;
  for (int64_t i0 = start; i0 < end; i0 += U) {
    int cs[U];
    float vs[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = i0 + u;
      const bool ok = i < end;
      cs[u] = ok ? assign[i] : -1;
      vs[u] = (ok && active) ? x[i * d + j] : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int c = cs[u];
      if (c < 0) continue;
      if (active) {
        if (SMEM) {
          acc_s[c * 32 + lane] = fadd(acc_s[c * 32 + lane], vs[u]);
        } else {
          float* p = my_sums + (int64_t)c * d + j;
          *p = fadd(*p, vs[u]);
        }
      }
      if (do_counts && lane == 0) cnt_s[c] += 1;
    }
  }
  __syncwarp();
  if (SMEM && active)
    for (int c = 0; c < k; ++c) my_sums[(int64_t)c * d + j] = acc_s[c * 32 + lane];
  if (do_counts)
    for (int c = lane; c < k; c += 32) local_counts[(int64_t)chunk * k + c] = cnt_s[c];
}

__global__ void k_kmeans_update(const float* __restrict__ x, int64_t n, int d, int k,
                                const float* __restrict__ local_sums,
                                const int32_t* __restrict__ local_counts, int64_t sample_offset,
                                int iteration, float* __restrict__ centroids, int64_t bx,
                                int64_t bs, int64_t bc, int64_t bcent) {
  x += blockIdx.y * bx;
  local_sums += blockIdx.y * bs;
  local_counts += blockIdx.y * bc;
  centroids += blockIdx.y * bcent;
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)k * d) return;
  const int c = (int)(e / d);
  const int j = (int)(e - (int64_t)c * d);
  float sum = 0.0f;  // kmeans.mojo:174-177 (zeroed) then :182-195
  int64_t count = 0;
  for (int ch = 0; ch < NUM_CHUNKS; ++ch) {
    count += local_counts[(int64_t)ch * k + c];
    sum = fadd(sum, local_sums[((int64_t)ch * k + c) * d + j]);
  }
  if (count > 0) {
    const float inv = __fdiv_rn(1.0f, __ll2float_rn(count));  // :202
    centroids[e] = fmul(sum, inv);
  } else {  // :211-220
    const int64_t src = (sample_offset + (int64_t)(iteration + 1) * k + c) % n;
    centroids[e] = x[src * d + j];
  }
}

__global__ void k_i32_to_i64(const int32_t* __restrict__ a, int64_t n, int64_t* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i];
}

}  // namespace

void launch_gather_rows(const float* x, int d, const int64_t* idx, int64_t count, float* out,
                        int batch, int64_t bx, int64_t bo, cudaStream_t s) {
  int64_t total = count * d;
  if (total == 0) return;
  dim3 grid((unsigned)((total + 255) / 256), (unsigned)batch);
  k_gather_rows<<<grid, 256, 0, s>>>(x, d, idx, count, out, bx, bo);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_kmeans_accumulate(const float* x, int64_t n, int d, int k, const int32_t* assign,
                              float* local_sums, int32_t* local_counts, int batch, int64_t bx,
                              int64_t ba, int64_t bs, int64_t bc, cudaStream_t s) {
  if (n == 0) return;
  dim3 grid(NUM_CHUNKS, (unsigned)((d + 31) / 32), (unsigned)batch);
  size_t smem_acc = (size_t)k * 32 * sizeof(float) + (size_t)k * sizeof(int);
  if (smem_acc <= 200 * 1024) {
    smem_limit(k_kmeans_accumulate<true>, smem_acc);
    k_kmeans_accumulate<true><<<grid, 32, smem_acc, s>>>(x, n, d, k, assign, local_sums,
                                                         local_counts, bx, ba, bs, bc);
  } else {
    size_t smem = (size_t)k * sizeof(int);
    MV_REQUIRE(smem <= 200 * 1024, MV_ERR_UNSUPPORTED, "k-means: k too large");
    smem_limit(k_kmeans_accumulate<false>, smem);
    k_kmeans_accumulate<false><<<grid, 32, smem, s>>>(x, n, d, k, assign, local_sums,
                                                      local_counts, bx, ba, bs, bc);
  }
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_kmeans_update(const float* x, int64_t n, int d, int k, const float* local_sums,
                          const int32_t* local_counts, int64_t sample_offset, int iteration,
                          float* centroids, int batch, int64_t bx, int64_t bs, int64_t bc,
                          int64_t bcent, cudaStream_t s) {
  int64_t total = (int64_t)k * d;
  dim3 grid((unsigned)((total + 255) / 256), (unsigned)batch);
  k_kmeans_update<<<grid, 256, 0, s>>>(x, n, d, k, local_sums, local_counts, sample_offset,
                                       iteration, centroids, bx, bs, bc, bcent);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_i32_to_i64(const int32_t* a, int64_t n, int64_t* out, cudaStream_t s) {
  if (n == 0) return;
  k_i32_to_i64<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, n, out);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
