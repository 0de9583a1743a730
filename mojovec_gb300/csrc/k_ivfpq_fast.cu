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

#include <algorithm>

namespace mv {
namespace {

constexpr int FT = 256;      // threads per CTA

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

// Coarse step of the fast form, one CTA per query: the nc smallest
// approximate (BF16 GEMM) distances by radix select, streamed over the nlist
// columns in chunks; their exact FP32 distances; the nprobe smallest, sorted
// ascending by (distance, list).
constexpr int CC_CHUNK = 4096;

__global__ void __launch_bounds__(FT)
    k_coarse_fast(const float* __restrict__ approx, int nlist, const float* __restrict__ q, int d,
                  const float* __restrict__ cent, int metric, int nc, int ncp, int nprobe,
                  int32_t* __restrict__ probes, float* __restrict__ term) {
  extern __shared__ __align__(16) unsigned char smraw[];
  uint64_t* keys = reinterpret_cast<uint64_t*>(smraw);  // CC_CHUNK + nc
  uint64_t* sel = keys + CC_CHUNK + nc;                 // ncp (power of two >= nc)
  float* qv = reinterpret_cast<float*>(sel + ncp);
  __shared__ RadixScratch rs;
  const int64_t row = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int j = threadIdx.x; j < d; j += FT) qv[j] = q[row * d + j];
  const float* arow = approx + row * (int64_t)nlist;
  int m = 0;
  for (int c0 = 0; c0 < nlist; c0 += CC_CHUNK) {
    const int len = min(CC_CHUNK, nlist - c0);
    for (int j = threadIdx.x; j < len; j += FT) keys[m + j] = make_key(arow[c0 + j], (uint32_t)(c0 + j));
    __syncthreads();
    const int r = block_radix_select<FT>(keys, m + len, nc, sel, rs);
    for (int j = threadIdx.x; j < r; j += FT) keys[j] = sel[j];
    __syncthreads();
    m = r;
  }
  // exact FP32 distances of the nc candidates
  for (int c = warp; c < ncp; c += FT / 32) {
    uint64_t out = KEY_NONE - (uint64_t)c;  // distinct padding keys sort last
    if (c < m) {
      const uint32_t list = key_id(keys[c]);
      const float* cp = cent + (int64_t)list * d;
      float acc = 0.0f;
      for (int j = lane; j < d; j += 32) {
        if (metric == MV_METRIC_L2) {
          const float df = qv[j] - cp[j];
          acc = fmaf(df, df, acc);
        } else {
          acc = fmaf(qv[j], cp[j], acc);
        }
      }
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      out = make_key(metric == MV_METRIC_L2 ? acc : -acc, list);
    }
    if (lane == 0) sel[c] = out;
  }
  __syncthreads();
  block_bitonic_sort(sel, ncp);
  for (int p = threadIdx.x; p < nprobe; p += FT) {
    const uint64_t key = p < m ? sel[p] : KEY_NONE;
    const bool ok = p < m;
    probes[row * nprobe + p] = ok ? (int32_t)key_id(key) : -1;
    term[row * nprobe + p] = ok ? key_dist(key) : 0.0f;
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

// ADC scan, one CTA per query. Candidate keys (distance, CSR position)
// are staged contiguously in shared memory; whenever the next chunk would
// overflow the staging area, and once at the end, a radix select keeps the R
// smallest. The shortlist is written unsorted (the rerank orders it), or
// sorted when it is the final answer.
__global__ void __launch_bounds__(FT) k_ivfpq_scan_fast(FastScanArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int M = a.M, d = a.d, dsub = d / M;
  float* lut = reinterpret_cast<float*>(smraw);
  float* qv = lut + M * 256;
  uint64_t* cand =
      reinterpret_cast<uint64_t*>(smraw + (((size_t)(M * 256 + d) * 4 + 15) & ~size_t(15)));
  uint64_t* outb = cand + a.cap;  // R (padded to a power of two when sorting)
  __shared__ RadixScratch rs;
  const int64_t row = blockIdx.x;
  for (int j = threadIdx.x; j < d; j += FT) qv[j] = a.q[row * d + j];
  __syncthreads();
  const float scale = a.metric == MV_METRIC_L2 ? -2.0f : -1.0f;
  for (int e = threadIdx.x; e < M * 256; e += FT) {
    const int mm = e >> 8, kk = e & 255;
    const float* c = a.pq + ((int64_t)mm * 256 + kk) * dsub;
    const float* x = qv + mm * dsub;
    float dot = 0.0f;
    for (int t = 0; t < dsub; ++t) dot = fmaf(x[t], c[t], dot);
    lut[e] = scale * dot;
  }
  __syncthreads();
  const int chunk = a.cap - a.R;
  int m = 0;
  for (int p = 0; p < a.nprobe; ++p) {
    const int list = a.probes[row * a.nprobe + p];
    if (list < 0) continue;
    const int64_t off = a.list_off[list];
    const int64_t ls = a.list_off[list + 1] - off;
    const float t1 = a.term[row * a.nprobe + p];
    for (int64_t j0 = 0; j0 < ls; j0 += chunk) {
      const int len = (int)min((int64_t)chunk, ls - j0);
      if (m + len > a.cap) {
        const int r = block_radix_select<FT>(cand, m, a.R, outb, rs);
        for (int j = threadIdx.x; j < r; j += FT) cand[j] = outb[j];
        __syncthreads();
        m = r;
      }
      for (int j = threadIdx.x; j < len; j += FT) {
        const int64_t pos = off + j0 + j;
        float acc = t1 + (a.vterm ? a.vterm[pos] : 0.0f);
        acc = adc_fast(lut, a.codes + pos * M, M, acc);
        cand[m + j] = make_key(acc, (uint32_t)pos);
      }
      m += len;
      __syncthreads();
    }
  }
  const int r = block_radix_select<FT>(cand, m, a.R, outb, rs);
  if (a.sorted) {
    for (int j = r + threadIdx.x; j < a.Rp; j += FT) outb[j] = KEY_NONE;
    __syncthreads();
    block_bitonic_sort(outb, a.Rp);
  }
  for (int i = threadIdx.x; i < a.R; i += FT) a.out_keys[row * a.R + i] = i < r ? outb[i] : KEY_NONE;
}

// Exact FP32 rerank of the shortlist against the raw rows (CSR order), one
// CTA per query: a warp per candidate row (float4 loads), radix select of
// the k smallest (distance, id), sorted.
__global__ void __launch_bounds__(FT) k_rerank_fast(RerankArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int d = a.d;
  float* qv = reinterpret_cast<float*>(smraw);
  uint64_t* ck = reinterpret_cast<uint64_t*>(smraw + (((size_t)d * 4 + 15) & ~size_t(15)));
  uint64_t* outb = ck + a.R;  // kp (power of two >= k)
  __shared__ RadixScratch rs;
  const int64_t row = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int j = threadIdx.x; j < d; j += FT) qv[j] = a.q[row * d + j];
  __syncthreads();
  const uint64_t* cand = a.cand + row * a.R;
  for (int c = warp; c < a.R; c += FT / 32) {
    const uint64_t key = cand[c];
    uint64_t out = KEY_NONE - (uint64_t)c;  // distinct keys for empty slots
    if (key != KEY_NONE) {
      const uint32_t pos = key_id(key);
      const float* x = a.raw + (int64_t)pos * d;
      float acc = 0.0f;
      if ((d & 3) == 0) {
        for (int j = lane * 4; j < d; j += 128) {
          const float4 v = *reinterpret_cast<const float4*>(x + j);
          if (a.metric == MV_METRIC_L2) {
            const float d0 = qv[j] - v.x, d1 = qv[j + 1] - v.y, d2 = qv[j + 2] - v.z,
                        d3 = qv[j + 3] - v.w;
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
            const float df = qv[j] - x[j];
            acc = fmaf(df, df, acc);
          } else {
            acc = fmaf(qv[j], x[j], acc);
          }
        }
      }
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      out = make_key(a.metric == MV_METRIC_L2 ? acc : -acc, a.ids[pos]);
    }
    if (lane == 0) ck[c] = out;
  }
  __syncthreads();
  const int r = block_radix_select<FT>(ck, a.R, a.k, outb, rs);
  for (int j = r + threadIdx.x; j < a.kp; j += FT) outb[j] = KEY_NONE;
  __syncthreads();
  block_bitonic_sort(outb, a.kp);
  for (int i = threadIdx.x; i < a.k; i += FT) {
    const uint64_t key = outb[i];
    float dd = 1e38f;
    int64_t ll = -1;
    if (key < KEY_NONE - (uint64_t)a.R) {  // padding keys are the top R values
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
  smem_limit(kernel, bytes);
}

}  // namespace

void launch_vec_terms(const int64_t* off, int nlist, const uint8_t* codes, const float* pq,
                      const float* cent, int d, int M, float* out, cudaStream_t s) {
  k_vec_terms<<<nlist, 128, 0, s>>>(off, codes, pq, cent, d, M, out);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_coarse_fast(const float* approx, int64_t nq, int nlist, const float* q, int d,
                        const float* cent, int metric, int nc, int nprobe, int32_t* probes,
                        float* term, cudaStream_t s) {
  if (nq == 0) return;
  const int ncp = next_pow2(nc);
  const size_t smem = (size_t)(CC_CHUNK + nc + ncp) * 8 + (size_t)d * 4;
  MV_REQUIRE(smem <= 200 * 1024, MV_ERR_UNSUPPORTED, "coarse select: nprobe or d too large");
  smem_attr(k_coarse_fast, smem);
  k_coarse_fast<<<(unsigned)nq, FT, smem, s>>>(approx, nlist, q, d, cent, metric, nc, ncp, nprobe,
                                                probes, term);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

int fast_scan_cap(int R) { return std::max(3072, 2 * R + 1024); }

void launch_ivfpq_scan_fast(FastScanArgs a, cudaStream_t s) {
  if (a.nq == 0) return;
  a.cap = fast_scan_cap(a.R);
  a.Rp = next_pow2(a.R);
  const size_t smem = (((size_t)(a.M * 256 + a.d) * 4 + 15) & ~size_t(15)) +
                      (size_t)(a.cap + a.Rp) * 8;
  MV_REQUIRE(smem <= 220 * 1024, MV_ERR_UNSUPPORTED, "fast IVF-PQ scan: M, d or shortlist too large");
  smem_attr(k_ivfpq_scan_fast, smem);
  k_ivfpq_scan_fast<<<(unsigned)a.nq, FT, smem, s>>>(a);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_rerank_fast(RerankArgs a, cudaStream_t s) {
  if (a.nq == 0) return;
  a.kp = next_pow2(a.k);
  const size_t smem = (((size_t)a.d * 4 + 15) & ~size_t(15)) + (size_t)(a.R + a.kp) * 8;
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
