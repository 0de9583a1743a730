// Fast-form IVF-PQ kernels (judged on recall against an FP64 ground truth,
// not on bit parity).
//
// The plain form rebuilds the residual LUT ||(q - c)_m - C[m][k]||^2 for
// every probed list (index/index_ivf_pq.mojo:306-315), 256 * d MACs per
// (query, list). The fast form expands the same squared distance as
//   ||q - c - y||^2 = ||q - c||^2 + (||y||^2 + 2 <c, y>) - 2 <q, y>
// with y the PQ reconstruction of the residual, so that
//   * ||q - c||^2 comes from the coarse step (exact FP32 recheck),
//   * ||y||^2 + 2<c, y> is one FP32 term per stored vector, computed when the
//     lists change (k_vec_terms),
//   * -2 <q_m, C[m][k]> is one M x 256 table per query, built once per query
//     in shared memory instead of once per probe.
// For the inner product the index distance is -<q, c> - sum_m <q_m, y_m>
// (index_ivf_pq.mojo:316-341) and the per-vector term is zero.
//
// The ADC scan keeps a shortlist of R candidates per query (BlockTopK over
// (distance, CSR position) keys); k_rerank_fast then computes exact FP32
// distances to the raw rows of the shortlist and selects the final k.
#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_fast.h"
#include "mv_select.cuh"

namespace mv {
namespace {

constexpr int FT = 256;      // threads per CTA
constexpr int FBUF = 512;    // BlockTopK buffer

__global__ void k_vec_terms(const int64_t* __restrict__ off, const uint8_t* __restrict__ codes,
                            const float* __restrict__ pq, const float* __restrict__ cent, int d,
                            int M, float* __restrict__ out) {
  const int list = blockIdx.x;
  const int dsub = d / M;
  const float* c = cent + (int64_t)list * d;
  for (int64_t e = off[list] + threadIdx.x; e < off[list + 1]; e += blockDim.x) {
    const uint8_t* code = codes + e * M;
    float s = 0.0f;
    for (int m = 0; m < M; ++m) {
      const float* y = pq + ((int64_t)m * 256 + code[m]) * dsub;
      const float* cm = c + m * dsub;
      for (int t = 0; t < dsub; ++t) s = fmaf(y[t], fmaf(2.0f, cm[t], y[t]), s);
    }
    out[e] = s;
  }
}

// Exact FP32 distances of a query to its candidate lists and the final
// top-nprobe (ascending (distance, list)). One CTA of 128 threads per query.
__global__ void __launch_bounds__(128)
    k_coarse_recheck(const float* __restrict__ q, int d, const float* __restrict__ cent,
                     int metric, const uint64_t* __restrict__ cand, int nc, int nprobe,
                     int32_t* __restrict__ probes, float* __restrict__ term) {
  extern __shared__ uint64_t ks[];  // nc keys
  const int64_t row = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float* qp = q + row * d;
  for (int c = warp; c < nc; c += 4) {
    const uint64_t key = cand[row * nc + c];
    uint64_t out = KEY_NONE;
    if (key != KEY_NONE) {
      const uint32_t list = key_id(key);
      const float* cp = cent + (int64_t)list * d;
      float acc = 0.0f;
      for (int j = lane; j < d; j += 32) {
        if (metric == MV_METRIC_L2) {
          float df = qp[j] - cp[j];
          acc = fmaf(df, df, acc);
        } else {
          acc = fmaf(qp[j], cp[j], acc);
        }
      }
      for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
      out = make_key(metric == MV_METRIC_L2 ? acc : -acc, list);
    }
    if (lane == 0) ks[c] = out;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nc; c += 128) {
    const uint64_t key = ks[c];
    int rank = 0;
    for (int j = 0; j < nc; ++j) rank += ks[j] < key;
    if (rank < nprobe) {
      probes[row * nprobe + rank] = key == KEY_NONE ? -1 : (int32_t)key_id(key);
      term[row * nprobe + rank] = key == KEY_NONE ? 0.0f : key_dist(key);
    }
  }
}

__device__ __forceinline__ float adc_fast(const float* lut, const uint8_t* code, int M, float acc) {
  if ((M & 15) == 0) {
    for (int m0 = 0; m0 < M; m0 += 16) {
      const uint4 v = *reinterpret_cast<const uint4*>(code + m0);
      const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc += lut[((m0 + 4 * i + b) << 8) + ((w[i] >> (8 * b)) & 255u)];
    }
  } else if ((M & 7) == 0) {
    for (int m0 = 0; m0 < M; m0 += 8) {
      const uint2 v = *reinterpret_cast<const uint2*>(code + m0);
      const uint32_t w[2] = {v.x, v.y};
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc += lut[((m0 + 4 * i + b) << 8) + ((w[i] >> (8 * b)) & 255u)];
    }
  } else {
    for (int m = 0; m < M; ++m) acc += lut[(m << 8) + code[m]];
  }
  return acc;
}

__global__ void __launch_bounds__(FT) k_ivfpq_scan_fast(FastScanArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int M = a.M, d = a.d, dsub = d / M;
  float* lut = reinterpret_cast<float*>(smraw);
  float* qv = lut + M * 256;
  uint64_t* keys =
      reinterpret_cast<uint64_t*>(smraw + (((size_t)(M * 256 + d) * 4 + 15) & ~size_t(15)));
  __shared__ int cnt;
  __shared__ uint64_t thr;
  const int64_t row = blockIdx.x;
  for (int j = threadIdx.x; j < d; j += FT) qv[j] = a.q[row * d + j];
  BlockTopK sel;
  sel.init(keys, &cnt, &thr, a.R, FBUF);
  const float scale = a.metric == MV_METRIC_L2 ? -2.0f : -1.0f;
  for (int e = threadIdx.x; e < M * 256; e += FT) {
    const int m = e >> 8, kk = e & 255;
    const float* c = a.pq + ((int64_t)m * 256 + kk) * dsub;
    const float* x = qv + m * dsub;
    float dot = 0.0f;
    for (int t = 0; t < dsub; ++t) dot = fmaf(x[t], c[t], dot);
    lut[e] = scale * dot;
  }
  __syncthreads();
  for (int p = 0; p < a.nprobe; ++p) {
    const int list = a.probes[row * a.nprobe + p];
    if (list < 0) continue;
    const int64_t off = a.list_off[list];
    const int64_t ls = a.list_off[list + 1] - off;
    const float t1 = a.term[row * a.nprobe + p];
    for (int64_t j0 = 0; j0 < ls; j0 += FT) {
      const int64_t j = j0 + threadIdx.x;
      if (j < ls) {
        const int64_t pos = off + j;
        float acc = t1 + (a.vterm ? a.vterm[pos] : 0.0f);
        acc = adc_fast(lut, a.codes + pos * M, M, acc);
        sel.push(make_key(acc, (uint32_t)pos));
      }
      sel.end_round();
    }
  }
  sel.finish();
  for (int i = threadIdx.x; i < a.R; i += FT) a.out_keys[row * a.R + i] = keys[i];
}

// Exact FP32 rerank of the shortlist against the raw rows (CSR order).
__global__ void __launch_bounds__(FT) k_rerank_fast(RerankArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int d = a.d;
  float* qv = reinterpret_cast<float*>(smraw);
  float* cd = qv + d;                                   // R distances
  uint32_t* cp = reinterpret_cast<uint32_t*>(cd + a.R); // R positions
  uint64_t* keys = reinterpret_cast<uint64_t*>(
      smraw + (((size_t)(d + 2 * a.R) * 4 + 15) & ~size_t(15)));
  __shared__ int cnt;
  __shared__ uint64_t thr;
  const int64_t row = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int j = threadIdx.x; j < d; j += FT) qv[j] = a.q[row * d + j];
  BlockTopK sel;
  sel.init(keys, &cnt, &thr, a.k, FBUF);  // syncs (qv visible)
  for (int c = warp; c < a.R; c += FT / 32) {
    const uint64_t key = a.cand[row * a.R + c];
    float dist = 0.0f;
    uint32_t pos = 0xffffffffu;
    if (key != KEY_NONE) {
      pos = key_id(key);
      const float* x = a.raw + (int64_t)pos * d;
      float acc = 0.0f;
      if ((d & 3) == 0) {
        for (int j = lane * 4; j < d; j += 128) {
          const float4 v = *reinterpret_cast<const float4*>(x + j);
          if (a.metric == MV_METRIC_L2) {
            float d0 = qv[j] - v.x, d1 = qv[j + 1] - v.y, d2 = qv[j + 2] - v.z, d3 = qv[j + 3] - v.w;
            acc = fmaf(d0, d0, acc);
            acc = fmaf(d1, d1, acc);
            acc = fmaf(d2, d2, acc);
            acc = fmaf(d3, d3, acc);
          } else {
            acc = fmaf(qv[j], v.x, acc);
            acc = fmaf(qv[j + 1], v.y, acc);
            acc = fmaf(qv[j + 2], v.z, acc);
            acc = fmaf(qv[j + 3], v.w, acc);
          }
        }
      } else {
        for (int j = lane; j < d; j += 32) {
          if (a.metric == MV_METRIC_L2) {
            float df = qv[j] - x[j];
            acc = fmaf(df, df, acc);
          } else {
            acc = fmaf(qv[j], x[j], acc);
          }
        }
      }
      for (int s = 16; s > 0; s >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, s);
      dist = a.metric == MV_METRIC_L2 ? acc : -acc;
    }
    if (lane == 0) {
      cd[c] = dist;
      cp[c] = pos;
    }
  }
  __syncthreads();
  for (int c0 = 0; c0 < a.R; c0 += FT) {
    const int c = c0 + threadIdx.x;
    if (c < a.R && cp[c] != 0xffffffffu) sel.push(make_key(cd[c], a.ids[cp[c]]));
    sel.end_round();
  }
  sel.finish();
  for (int i = threadIdx.x; i < a.k; i += FT) {
    const uint64_t key = keys[i];
    float dd = 1e38f;
    int64_t ll = -1;
    if (key != KEY_NONE) {
      dd = key_dist(key);
      if (a.metric != MV_METRIC_L2) dd = -dd;
      ll = (int64_t)key_id(key);
    }
    a.out_d[row * a.k + i] = dd;
    a.out_l[row * a.k + i] = ll;
  }
}

// Shortlist without rerank: the first k keys (already sorted) -> results.
__global__ void k_short_to_results(const uint64_t* __restrict__ keys, int64_t nq, int R, int k,
                                   const uint32_t* __restrict__ ids, int metric,
                                   float* __restrict__ out_d, int64_t* __restrict__ out_l) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq * k) return;
  const int64_t r = i / k;
  const int j = (int)(i - r * k);
  const uint64_t key = keys[r * R + j];
  if (key == KEY_NONE) {
    out_d[i] = 1e38f;
    out_l[i] = -1;
  } else {
    const float dd = key_dist(key);
    out_d[i] = metric == MV_METRIC_L2 ? dd : -dd;
    out_l[i] = ids[key_id(key)];
  }
}

template <typename K>
void smem_attr(K kernel, size_t bytes) {
  if (bytes > 48 * 1024)
    MV_CHECK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

}  // namespace

void launch_vec_terms(const int64_t* off, int nlist, const uint8_t* codes, const float* pq,
                      const float* cent, int d, int M, float* out, cudaStream_t s) {
  k_vec_terms<<<nlist, 128, 0, s>>>(off, codes, pq, cent, d, M, out);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_coarse_recheck(const float* q, int64_t nq, int d, const float* cent, int metric,
                           const uint64_t* cand, int nc, int nprobe, int32_t* probes, float* term,
                           cudaStream_t s) {
  if (nq == 0) return;
  size_t smem = (size_t)nc * 8;
  MV_REQUIRE(smem <= 200 * 1024, MV_ERR_UNSUPPORTED, "coarse recheck: nprobe too large");
  smem_attr(k_coarse_recheck, smem);
  k_coarse_recheck<<<(unsigned)nq, 128, smem, s>>>(q, d, cent, metric, cand, nc, nprobe, probes, term);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_ivfpq_scan_fast(const FastScanArgs& a, cudaStream_t s) {
  if (a.nq == 0) return;
  size_t smem = (((size_t)(a.M * 256 + a.d) * 4 + 15) & ~size_t(15)) +
                (size_t)BlockTopK::smem_keys(a.R, FBUF) * 8;
  MV_REQUIRE(smem <= 220 * 1024, MV_ERR_UNSUPPORTED, "fast IVF-PQ scan: M, d or shortlist too large");
  smem_attr(k_ivfpq_scan_fast, smem);
  k_ivfpq_scan_fast<<<(unsigned)a.nq, FT, smem, s>>>(a);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_rerank_fast(const RerankArgs& a, cudaStream_t s) {
  if (a.nq == 0) return;
  size_t smem = (((size_t)(a.d + 2 * a.R) * 4 + 15) & ~size_t(15)) +
                (size_t)BlockTopK::smem_keys(a.k, FBUF) * 8;
  MV_REQUIRE(smem <= 220 * 1024, MV_ERR_UNSUPPORTED, "rerank: d or shortlist too large");
  smem_attr(k_rerank_fast, smem);
  k_rerank_fast<<<(unsigned)a.nq, FT, smem, s>>>(a);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_short_to_results(const uint64_t* keys, int64_t nq, int R, int k, const uint32_t* ids,
                             int metric, float* out_d, int64_t* out_l, cudaStream_t s) {
  const int64_t total = nq * k;
  if (total == 0) return;
  k_short_to_results<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(keys, nq, R, k, ids, metric,
                                                                     out_d, out_l);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
