// Certified exact nearest-centroid assignment.
//
// The reference assigns a row to its nearest centroid with FP32 distances in
// a fixed operation order (index/index_flat.mojo:292-310 with k = 1 for the
// coarse quantizer; clustering/kmeans.mojo:123-141 in k-means): the smallest
// distance, the smaller index on equal distances. Here the BF16 tensor-core
// top-k GEMM (k_umma_topk) proposes kc candidates per row, k_assign_certify
// recomputes the candidates with the reference's FP32 distance and keeps the
// best, and a rigorous bound on the BF16 ranking error decides whether any
// centroid outside the candidates could still be nearer. Rows the bound does
// not settle (and rows with NaN or huge distances) are listed for the exact
// SIMT argmin, so the result always equals the exact one.
//
// Bound (bx, by: the rows rounded to BF16, round to nearest, unit roundoff
// u = 2^-8; X = ||bx||, B = max over centroids of ||by||). The candidate key
// of centroid c is kd(c) = fl(||by||^2 - 2 acc), acc the tensor-core FP32 sum
// of the exact products bx_i * by_i, ||by||^2 summed in FP32:
//   | kd(c) - (||by||^2 - 2 bx.by) | <= (d + 1) 2^-23 B^2 + (d + 1) 2^-21 X B
// (each FP32 addition of the tensor core's sum taken as losing up to 2^-22
// of the sum of |products|; the code doubles that term). Rows or centroids
// with norms outside [1e-15, 1e150] are not certified.
// Every centroid outside the candidates has kd(c) >= K, the kc-th smallest
// candidate key (a per-segment heap or the shared threshold dropped it only
// below kc better keys that the candidates still hold, or beat). Then
//   L2: ||bx - by|| >= sqrt(X^2 + K - eps) and, as ||x - bx|| <= u ||x||,
//       ||x - y|| >= sqrt(X^2 + K - eps) - u (X + B) / (1 - u) = s,
//       and the reference distance is at least s^2 (1 - g), g = (d + 16) 2^-23
//       (FP32 sum of non-negative squares);
//   IP: x.y <= -K + (2u (1 + 2u) + (d + 1) 2^-21) X B, and the reference
//       distance -fl(x.y) >= K - (2u (1 + 2u) + (d + 1) 2^-21 + g (1 + 3u)) X B.
// A row is settled when that lower bound exceeds the best candidate's
// reference distance (strictly, so ties cannot hide outside).
#include <cuda_bf16.h>

#include "mv_exact.cuh"
#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"

namespace mv {
namespace {

// B^2 upper bound: max of the FP32 norms of the BF16 rows, with the FP32
// summation error added.
__global__ void k_max_norm(const float* __restrict__ norms, int n, int d, double* __restrict__ out) {
  __shared__ double part[32];
  double m = 0.0;
  bool bad = false;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float v = norms[i];
    if (!(v <= 3.0e38f)) bad = true;  // NaN or inf
    m = fmax(m, (double)v);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  bad = __any_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = bad ? -1.0 : m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    bool anybad = false;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      if (part[w] < 0.0) anybad = true;
      r = fmax(r, part[w]);
    }
    *out = anybad ? -1.0 : r * (1.0 + (d + 1) * 0x1p-23);
  }
}

__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}

// One warp per row.
template <bool IP>
__global__ void k_assign_certify(const float* __restrict__ x, int64_t n, int d,
                                 const float* __restrict__ cent, int nlist,
                                 const uint64_t* __restrict__ cand, int ncand, int kc,
                                 const double* __restrict__ bmax2, int32_t* __restrict__ assign,
                                 float* __restrict__ mind, int64_t* __restrict__ flagged,
                                 int* __restrict__ nflag) {
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float* xr = x + row * d;
  const uint64_t* ck = cand + row * ncand;
  float best = __int_as_float(0x7f800000);
  int bi = 0x7fffffff;
  bool bad = false;
  int valid = 0;
  for (int c = lane; c < ncand; c += 32) {
    const uint64_t key = ck[c];
    if (key == KEY_NONE) continue;
    const uint32_t ci = key_id(key);
    if (ci >= (uint32_t)nlist) continue;
    ++valid;
    const float* yr = cent + (int64_t)ci * d;
    const float r = IP ? -ip_simd<8>(xr, yr, d) : l2_simd<8>(xr, yr, d);
    if (r != r) bad = true;
    if (r < best || (r == best && (int)ci < bi)) {
      best = r;
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
    valid += __shfl_xor_sync(0xffffffffu, valid, o);
  }
  bad = __any_sync(0xffffffffu, bad);
  bool ok = !bad && bi != 0x7fffffff && best < 1e38f;
  if (ok && valid < nlist) {
    // K: the kc-th smallest candidate key
    uint64_t prev = 0;
    for (int t = 0; t < kc; ++t) {
      uint64_t m = KEY_NONE;
      for (int c = lane; c < ncand; c += 32) {
        const uint64_t key = ck[c];
        if (key == KEY_NONE || key_id(key) >= (uint32_t)nlist) continue;
        if ((t == 0 || key > prev) && key < m) m = key;
      }
      prev = warp_min_u64(m);
    }
    // X^2 = ||bx||^2 (exact in double)
    double xs = 0.0;
    for (int j = lane; j < d; j += 32) {
      const double b = (double)__bfloat162float(__float2bfloat16_rn(xr[j]));
      xs = fma(b, b, xs);
    }
    for (int o = 16; o > 0; o >>= 1) xs += __shfl_xor_sync(0xffffffffu, xs, o);
    const double B2 = *bmax2;
    if (valid < kc || prev == KEY_NONE || !(B2 >= 1e-30) || !(xs >= 1e-30 && xs <= 1e300)) {
      ok = false;
    } else {
      const double K = (double)key_dist(prev);
      const double X = sqrt(xs), B = sqrt(B2);
      const double u = 0x1p-8;
      const double g = (d + 16) * 0x1p-23;
      const double ea = (d + 1) * 0x1p-20;  // twice the tensor-core accumulation bound
      const double eabs = d * 1e-36;         // products below FP32's normal range
      double lower;
      if (IP) {
        lower = K - (2.0 * u * (1.0 + 2.0 * u) + ea + g * (1.0 + 3.0 * u)) * X * B * 1.01 - eabs;
      } else {
        const double eps = ((d + 1) * 0x1p-23 * B2 + ea * X * B) * 1.01 + eabs;
        const double sb = X * X + K - eps;
        const double s = (sb > 0.0 ? sqrt(sb) : 0.0) - u * (X + B) / (1.0 - u) * 1.01;
        lower = s > 0.0 ? s * s * (1.0 - g) : -1.0;
      }
      ok = lower > (double)best;
    }
  }
  if (lane == 0) {
    assign[row] = bi == 0x7fffffff ? 0 : bi;
    if (mind) mind[row] = best;
    if (!ok) flagged[atomicAdd(nflag, 1)] = row;
  }
}

__global__ void k_scatter_assign(const int32_t* __restrict__ sub, const float* __restrict__ sub_d,
                                 const int64_t* __restrict__ idx, int64_t count,
                                 int32_t* __restrict__ assign, float* __restrict__ mind) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  assign[idx[i]] = sub[i];
  if (mind) mind[idx[i]] = sub_d[i];
}

}  // namespace

void launch_max_norm(const float* norms, int n, int d, double* out, cudaStream_t s) {
  k_max_norm<<<1, 1024, 0, s>>>(norms, n, d, out);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_assign_certify(const float* x, int64_t n, int d, const float* cent, int nlist, int metric,
                           const uint64_t* cand, int ncand, int kc, const double* bmax2,
                           int32_t* assign, float* mind, int64_t* flagged, int* nflag,
                           cudaStream_t s) {
  if (n == 0) return;
  const unsigned grid = (unsigned)((n + 7) / 8);
  if (metric == MV_METRIC_IP)
    k_assign_certify<true><<<grid, 256, 0, s>>>(x, n, d, cent, nlist, cand, ncand, kc, bmax2,
                                                       assign, mind, flagged, nflag);
  else
    k_assign_certify<false><<<grid, 256, 0, s>>>(x, n, d, cent, nlist, cand, ncand, kc, bmax2,
                                                        assign, mind, flagged, nflag);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_scatter_assign(const int32_t* sub, const float* sub_d, const int64_t* idx, int64_t count,
                           int32_t* assign, float* mind, cudaStream_t s) {
  if (count == 0) return;
  k_scatter_assign<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(sub, sub_d, idx, count, assign,
                                                                  mind);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
