// Plain (reference-exact) IVF-PQ kernels: per-query residual LUT + uint8
// ADC scan + k-select, PQ encoding and distance tables.
//
// k_ivfpq_scan_plain restates the per-query loop of IndexIVFPQ.search
// (index/index_ivf_pq.mojo:276-360). One CTA owns one query:
//   * L2: for each probed list, the residual q - c (:309-310) and its LUT
//     (ProductQuantizer.compute_distance_table, quantization/pq.mojo:252-292)
//     are built in shared memory;
//   * IP: the LUT is built once from q (:288-293) and each list adds
//     -inner_product_simd[8](q, c) (:316-324);
//   * ADC: dist = coarse + sum_m LUT[m][code[m]] left to right (:336-341),
//     filter skip (:328-334), canonical top-k via BlockTopK.
// Codes are read with 16/8/4-byte vector loads straight from the CSR lists
// (coalesced across the CTA: consecutive threads take consecutive vectors).
#include "mv_exact.cuh"
#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"

namespace mv {
namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_BUF = 512;

__device__ __forceinline__ float adc_sum(const float* lut, const uint8_t* code, int M, float init) {
  float dist = init;
  if ((M & 15) == 0) {
    for (int m0 = 0; m0 < M; m0 += 16) {
      uint4 v = *reinterpret_cast<const uint4*>(code + m0);
      uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          int m = m0 + q * 4 + b;
          dist = fadd(dist, lut[(m << 8) + ((w[q] >> (8 * b)) & 255u)]);
        }
    }
  } else if ((M & 7) == 0) {
    for (int m0 = 0; m0 < M; m0 += 8) {
      uint2 v = *reinterpret_cast<const uint2*>(code + m0);
      uint32_t w[2] = {v.x, v.y};
#pragma unroll
      for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          int m = m0 + q * 4 + b;
          dist = fadd(dist, lut[(m << 8) + ((w[q] >> (8 * b)) & 255u)]);
        }
    }
  } else {
    for (int m = 0; m < M; ++m) dist = fadd(dist, lut[(m << 8) + code[m]]);
  }
  return dist;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_ivfpq_scan_plain(IvfpqScanArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int M = a.M, d = a.d, dsub = a.dsub;
  float* lut = reinterpret_cast<float*>(smraw);
  float* vec = lut + M * 256;
  float* res = vec + d;
  uint64_t* keys = reinterpret_cast<uint64_t*>(smraw + (((size_t)(M * 256 + 2 * d) * 4 + 15) & ~size_t(15)));
  __shared__ int cnt;
  __shared__ uint64_t thr;
  __shared__ float coarse_s;
  const int64_t q = blockIdx.x;
  const float* qp = a.q + q * d;
  for (int j = threadIdx.x; j < d; j += SCAN_THREADS) vec[j] = qp[j];
  BlockTopK sel;
  sel.init(keys, &cnt, &thr, a.k, SCAN_BUF);  // syncs
  const bool ip = (a.metric == MV_METRIC_IP);
  if (ip) {  // LUT from q (index_ivf_pq.mojo:288-293)
    for (int e = threadIdx.x; e < M * 256; e += SCAN_THREADS) {
      int m = e >> 8, kk = e & 255;
      lut[e] = pq_sub_negip(vec + m * dsub, a.pq + ((int64_t)m * 256 + kk) * dsub, dsub);
    }
  }
  __syncthreads();
  for (int p = 0; p < a.nprobe; ++p) {
    const int list = a.probes[q * a.nprobe + p];
    if (list < 0) continue;
    const int64_t off = a.list_off[list];
    const int64_t ls = a.list_off[list + 1] - off;
    if (ls == 0) continue;
    const float* cp = a.centroids + (int64_t)list * d;
    float coarse = 0.0f;
    if (!ip) {
      for (int j = threadIdx.x; j < d; j += SCAN_THREADS) res[j] = fsub(vec[j], cp[j]);
      __syncthreads();
      for (int e = threadIdx.x; e < M * 256; e += SCAN_THREADS) {
        int m = e >> 8, kk = e & 255;
        lut[e] = pq_sub_l2(res + m * dsub, a.pq + ((int64_t)m * 256 + kk) * dsub, dsub);
      }
      __syncthreads();
    } else {
      if (threadIdx.x == 0) coarse_s = -ip_simd<8>(vec, cp, d);
      __syncthreads();
      coarse = coarse_s;
    }
    for (int64_t j0 = 0; j0 < ls; j0 += SCAN_THREADS) {
      const int64_t j = j0 + threadIdx.x;
      if (j < ls) {
        const uint32_t id = a.ids[off + j];
        if (!(a.filter && (int64_t)id < a.filter_len && a.filter[id] != 0)) {
          float dist = adc_sum(lut, a.codes + (off + j) * M, M, coarse);
          sel.push(make_key(dist, id));
        }
      }
      sel.end_round();
    }
  }
  sel.finish();
  for (int i = threadIdx.x; i < a.k; i += SCAN_THREADS) {
    uint64_t key = keys[i];
    float dd;
    int64_t ll;
    if (key == KEY_NONE) {  // index_ivf_pq.mojo:284-286 prefill
      dd = 1e38f;
      ll = -1;
    } else {
      dd = key_dist(key);
      if (ip) dd = -dd;  // :357-360
      ll = (int64_t)key_id(key);
    }
    a.out_d[q * a.k + i] = dd;
    a.out_l[q * a.k + i] = ll;
  }
}

__global__ void k_residuals(const float* __restrict__ x, int64_t n, int d,
                            const float* __restrict__ cent, int nlist,
                            const int32_t* __restrict__ assign, float* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * d) return;
  int64_t r = i / d;
  int j = (int)(i - r * d);
  int l = assign[r];
  if (l < 0 || l >= nlist) l = 0;  // index_ivf_pq.mojo:182-184
  out[i] = fsub(x[i], cent[(int64_t)l * d + j]);
}

// One warp per subspace m, lanes over vectors; codewords are read with
// warp-uniform (broadcast) loads.
__global__ void k_pq_encode(const float* __restrict__ x, int64_t n, int d, int M,
                            const float* __restrict__ pq, uint8_t* __restrict__ codes) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  const int dsub = d / M;
  const int64_t i = (int64_t)blockIdx.x * 32 + lane;
  for (int m = warp; m < M; m += nwarps) {
    if (i >= n) continue;
    const float* sub = x + i * d + m * dsub;
    const float* cm = pq + (int64_t)m * 256 * dsub;
    float min_dist = 1e38f;
    int best = -1;
    for (int kk = 0; kk < 256; ++kk) {
      float dist = pq_sub_l2(sub, cm + kk * dsub, dsub);
      if (dist < min_dist) {  // strict `<` (pq.mojo:215-217)
        min_dist = dist;
        best = kk;
      }
    }
    codes[i * M + m] = (uint8_t)best;
  }
}

__global__ void k_pq_tables(const float* __restrict__ x, int d, int M, const float* __restrict__ pq,
                            int metric, float* __restrict__ out) {
  const int64_t q = blockIdx.x;
  const int dsub = d / M;
  const float* qp = x + q * d;
  for (int e = threadIdx.x; e < M * 256; e += blockDim.x) {
    int m = e >> 8, kk = e & 255;
    const float* c = pq + ((int64_t)m * 256 + kk) * dsub;
    out[q * M * 256 + e] = metric == MV_METRIC_L2 ? pq_sub_l2(qp + m * dsub, c, dsub)
                                                  : pq_sub_negip(qp + m * dsub, c, dsub);
  }
}

__global__ void k_split_subspaces(const float* __restrict__ x, int64_t n, int d, int M,
                                  float* __restrict__ out) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * d) return;
  int64_t i = e / d;
  int j = (int)(e - i * d);
  int dsub = d / M;
  int m = j / dsub, t = j - m * dsub;
  out[((int64_t)m * n + i) * dsub + t] = x[e];
}

}  // namespace

void launch_ivfpq_scan_plain(const IvfpqScanArgs& a, cudaStream_t s) {
  if (a.nq == 0) return;
  size_t smem = (((size_t)(a.M * 256 + 2 * a.d) * 4 + 15) & ~size_t(15)) +
                (size_t)BlockTopK::smem_keys(a.k, SCAN_BUF) * 8;
  MV_REQUIRE(smem <= 220 * 1024, MV_ERR_UNSUPPORTED, "IVF-PQ scan: M, d or k too large");
  MV_REQUIRE(a.nq <= 0x7fffffff, MV_ERR_UNSUPPORTED, "too many queries");
  smem_limit(k_ivfpq_scan_plain, smem);
  k_ivfpq_scan_plain<<<(unsigned)a.nq, SCAN_THREADS, smem, s>>>(a);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_residuals(const float* x, int64_t n, int d, const float* centroids, int nlist,
                      const int32_t* assign, float* out, cudaStream_t s) {
  int64_t total = n * d;
  if (total == 0) return;
  k_residuals<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(x, n, d, centroids, nlist, assign, out);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_pq_encode(const float* x, int64_t n, int d, int M, const float* pq, uint8_t* codes,
                      cudaStream_t s) {
  if (n == 0) return;
  int warps = M < 8 ? M : 8;
  k_pq_encode<<<(unsigned)((n + 31) / 32), 32 * warps, 0, s>>>(x, n, d, M, pq, codes);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_pq_tables(const float* x, int64_t nq, int d, int M, const float* pq, int metric,
                      float* out, cudaStream_t s) {
  if (nq == 0) return;
  k_pq_tables<<<(unsigned)nq, 256, 0, s>>>(x, d, M, pq, metric, out);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_split_subspaces(const float* x, int64_t n, int d, int M, float* out, cudaStream_t s) {
  int64_t total = n * d;
  if (total == 0) return;
  k_split_subspaces<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(x, n, d, M, out);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
