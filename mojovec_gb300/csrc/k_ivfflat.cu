// IVF-Flat scan (index/index_ivf_flat.mojo:176-243): for each probed list,
// the exact FP32 distance of every stored row to the query, L2 as
// l2_distance_simd[8] and IP as -inner_product_simd[4] (the reference's two
// widths), into the canonical top-k (distance, then the smaller id); tail
// 1e38 / -1 and IP un-negated (:199-203, :241-243).
//
// One CTA of FT threads per query (several CTAs per SM, so one CTA's loads
// overlap another's arithmetic). Candidate rows are staged through shared
// memory in tiles of up to FT rows, each warp reading 8 rows at a time with
// coalesced (float4 where d allows) loads all issued before the stores, at a
// row stride of d + 1 floats so that thread t
// reading row t touches its own bank; thread t then computes row t's
// distance with the same per-thread, in-order routine as the oracle.
#include "mv_exact.cuh"
#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"

namespace mv {
namespace {

constexpr int FT = 64;
constexpr int TOP_BUF = 256;

template <bool IP>
__global__ void __launch_bounds__(FT)
    k_ivfflat_scan(const float* __restrict__ q, int d, const int32_t* __restrict__ probes,
                   int nprobe, int nlist, const int64_t* __restrict__ list_off,
                   const float* __restrict__ rows, const uint32_t* __restrict__ ids, int tr, int k,
                   float* __restrict__ out_d, int64_t* __restrict__ out_l) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float* qs = reinterpret_cast<float*>(smraw);
  float* tile = qs + d;  // tr x (d + 1)
  uint64_t* keys =
      reinterpret_cast<uint64_t*>(smraw + (((size_t)(d + (size_t)tr * (d + 1)) * 4 + 15) & ~size_t(15)));
  __shared__ int cnt;
  __shared__ uint64_t thr;
  const int64_t row = blockIdx.x;
  for (int j = threadIdx.x; j < d; j += FT) qs[j] = q[row * d + j];
  BlockTopK sel;
  sel.init(keys, &cnt, &thr, k, TOP_BUF);  // syncs
  const int stride = d + 1;
  for (int p = 0; p < nprobe; ++p) {
    const int list = probes[row * nprobe + p];
    if (list < 0 || list >= nlist) continue;
    const int64_t off = list_off[list];
    const int64_t ls = list_off[list + 1] - off;
    for (int64_t j0 = 0; j0 < ls; j0 += tr) {
      const int nr = ls - j0 < tr ? (int)(ls - j0) : tr;
      __syncthreads();  // the previous tile is consumed
      const float* src = rows + (off + j0) * d;
      const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
      if ((d & 3) == 0) {
        // UR rows per warp per step: all of their loads are issued before
        // the stores, so each warp keeps UR row slices in flight.
        constexpr int UR = 8;
        for (int r0 = warp * UR; r0 < nr; r0 += (FT / 32) * UR) {
          for (int c4 = lane; c4 < (d >> 2); c4 += 32) {
            float4 v[UR];
#pragma unroll
            for (int u = 0; u < UR; ++u)
              v[u] = r0 + u < nr ? __ldg(reinterpret_cast<const float4*>(src + (int64_t)(r0 + u) * d) + c4)
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int u = 0; u < UR; ++u) {
              if (r0 + u < nr) {
                float* t = tile + (r0 + u) * stride + 4 * c4;
                t[0] = v[u].x;
                t[1] = v[u].y;
                t[2] = v[u].z;
                t[3] = v[u].w;
              }
            }
          }
        }
      } else {
        for (int r = warp; r < nr; r += FT / 32) {
          const float* sr = src + (int64_t)r * d;
          float* t = tile + r * stride;
          for (int c = lane; c < d; c += 32) t[c] = __ldg(sr + c);
        }
      }
      __syncthreads();
      for (int r0 = 0; r0 < nr; r0 += FT) {
        const int r = r0 + threadIdx.x;
        if (r < nr) {
          const float* bp = tile + r * stride;
          const float dist = IP ? -ip_simd<4>(qs, bp, d) : l2_simd<8>(qs, bp, d);
          sel.push(make_key(dist, ids[off + j0 + r]));
        }
        sel.end_round();
      }
    }
  }
  sel.finish();
  for (int i = threadIdx.x; i < k; i += FT) {
    const uint64_t key = keys[i];
    float dd = 1e38f;
    int64_t ll = -1;
    if (key != KEY_NONE) {
      dd = key_dist(key);
      if (IP) dd = -dd;
      ll = (int64_t)key_id(key);
    }
    out_d[row * k + i] = dd;
    out_l[row * k + i] = ll;
  }
}

// ---- List-major scan (k <= 32) ----------------------------------------
// The (query, probe) pairs are grouped by list on the device; one CTA takes
// a list and up to LM_QC of its queries, stages each tile of the list's rows
// once (as above) and computes every row's distance to each of those
// queries with the same per-thread routine, so the list is read once per
// LM_QC queries instead of once per query. Each (query, list) keeps its 32
// smallest keys in a warp's registers (sorted), its k smallest are written
// per (query, probe), and a warp per query merges its nprobe x k keys. The
// union of the per-list k smallest holds the query's k smallest keys, so the
// results equal the query-major scan's.
constexpr int LM_T = 64;   // threads per CTA = rows per tile
constexpr int LM_QC = 4;   // queries per CTA (measured: 2, 8 and 16 are slower)

__global__ void k_lm_count(const int32_t* __restrict__ probes, int64_t npairs, int nlist,
                           int* __restrict__ cnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npairs) return;
  const int L = probes[i];
  if (L >= 0 && L < nlist) atomicAdd(&cnt[L], 1);
}

// Exclusive scans of cnt (start[0..nlist]) and of ceil(cnt / qc)
// (istart[0..nlist]); one block of 1024 threads.
__global__ void __launch_bounds__(1024)
    k_lm_offsets(const int* __restrict__ cnt, int nlist, int qc, int64_t* __restrict__ start,
                 int* __restrict__ istart) {
  __shared__ long long ws1[32];
  __shared__ int ws2[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int per = (nlist + 1023) / 1024;
  const int b0 = min(nlist, t * per), b1 = min(nlist, b0 + per);
  long long s1 = 0;
  int s2 = 0;
  for (int L = b0; L < b1; ++L) {
    s1 += cnt[L];
    s2 += (cnt[L] + qc - 1) / qc;
  }
  long long i1 = s1;
  int i2 = s2;
  for (int o = 1; o < 32; o <<= 1) {
    const long long a = __shfl_up_sync(0xffffffffu, i1, o);
    const int b = __shfl_up_sync(0xffffffffu, i2, o);
    if (lane >= o) {
      i1 += a;
      i2 += b;
    }
  }
  if (lane == 31) {
    ws1[w] = i1;
    ws2[w] = i2;
  }
  __syncthreads();
  if (w == 0) {
    long long a = ws1[lane];
    int b = ws2[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const long long x = __shfl_up_sync(0xffffffffu, a, o);
      const int y = __shfl_up_sync(0xffffffffu, b, o);
      if (lane >= o) {
        a += x;
        b += y;
      }
    }
    ws1[lane] = a;
    ws2[lane] = b;
  }
  __syncthreads();
  long long base1 = (w ? ws1[w - 1] : 0) + i1 - s1;
  int base2 = (w ? ws2[w - 1] : 0) + i2 - s2;
  for (int L = b0; L < b1; ++L) {
    start[L] = base1;
    istart[L] = base2;
    base1 += cnt[L];
    base2 += (cnt[L] + qc - 1) / qc;
  }
  if (t == 1023) {
    start[nlist] = ws1[31];
    istart[nlist] = ws2[31];
  }
}

__global__ void k_lm_place(const int32_t* __restrict__ probes, int64_t npairs, int nlist,
                           const int64_t* __restrict__ start, int* __restrict__ cursor,
                           int32_t* __restrict__ pairs) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npairs) return;
  const int L = probes[i];
  if (L >= 0 && L < nlist) pairs[start[L] + atomicAdd(&cursor[L], 1)] = (int32_t)i;
}

template <bool IP>
__global__ void __launch_bounds__(LM_T)
    k_lm_scan(const float* __restrict__ q, int d, int P, const int64_t* __restrict__ list_off,
              const float* __restrict__ rows, const uint32_t* __restrict__ ids,
              const int* __restrict__ cnt, const int64_t* __restrict__ start,
              const int* __restrict__ istart, int nlist, const int32_t* __restrict__ pairs, int k,
              uint64_t* __restrict__ out_pk) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int stride = d + 1;
  float* qs = reinterpret_cast<float*>(smraw);  // LM_QC x d
  float* tile = qs + (size_t)LM_QC * d;          // LM_T x (d + 1)
  uint64_t* kk = reinterpret_cast<uint64_t*>(
      smraw + (((size_t)(LM_QC * d + (size_t)LM_T * stride) * 4 + 15) & ~size_t(15)));  // LM_QC x LM_T
  __shared__ int s_L, s_n;
  __shared__ int64_t s_pbase;
  const int b = blockIdx.x;
  if (threadIdx.x == 0) {
    int L = -1;
    if (b < istart[nlist]) {  // the list with istart[L] <= b < istart[L + 1]
      int lo = 0, hi = nlist - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (istart[mid] <= b) lo = mid;
        else hi = mid - 1;
      }
      L = lo;
      const int c = b - istart[L];
      s_pbase = start[L] + (int64_t)c * LM_QC;
      s_n = min(LM_QC, cnt[L] - c * LM_QC);
    }
    s_L = L;
  }
  __syncthreads();
  const int L = s_L;
  if (L < 0) return;  // uniform
  const int nqc = s_n;
  const int64_t pbase = s_pbase;
  for (int j = 0; j < nqc; ++j) {
    const int64_t qi = pairs[pbase + j] / P;
    for (int c = threadIdx.x; c < d; c += LM_T) qs[j * d + c] = q[qi * d + c];
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t best[LM_QC / 2];  // warp w keeps queries w, w + 2, ...
#pragma unroll
  for (int u = 0; u < LM_QC / 2; ++u) best[u] = KEY_NONE;
  const int64_t off = list_off[L];
  const int64_t ls = list_off[L + 1] - off;
  for (int64_t r0 = 0; r0 < ls; r0 += LM_T) {
    const int nr = ls - r0 < LM_T ? (int)(ls - r0) : LM_T;
    __syncthreads();  // the previous tile and keys are consumed
    const float* src = rows + (off + r0) * d;
    if ((d & 3) == 0) {
      constexpr int UR = 8;
      for (int q0 = warp * UR; q0 < nr; q0 += (LM_T / 32) * UR) {
        for (int c4 = lane; c4 < (d >> 2); c4 += 32) {
          float4 v[UR];
#pragma unroll
          for (int u = 0; u < UR; ++u)
            v[u] = q0 + u < nr ? __ldg(reinterpret_cast<const float4*>(src + (int64_t)(q0 + u) * d) + c4)
                               : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
          for (int u = 0; u < UR; ++u) {
            if (q0 + u < nr) {
              float* t = tile + (q0 + u) * stride + 4 * c4;
              t[0] = v[u].x;
              t[1] = v[u].y;
              t[2] = v[u].z;
              t[3] = v[u].w;
            }
          }
        }
      }
    } else {
      for (int r = warp; r < nr; r += LM_T / 32) {
        const float* sr = src + (int64_t)r * d;
        float* t = tile + r * stride;
        for (int c = lane; c < d; c += 32) t[c] = __ldg(sr + c);
      }
    }
    __syncthreads();
    const int r = threadIdx.x;
    if (r < nr) {
      const float* bp = tile + r * stride;
      const uint32_t id = ids[off + r0 + r];
      for (int j = 0; j < nqc; ++j) {
        const float dist = IP ? -ip_simd<4>(qs + j * d, bp, d) : l2_simd<8>(qs + j * d, bp, d);
        kk[j * LM_T + r] = make_key(dist, id);
      }
    } else {
      for (int j = 0; j < nqc; ++j) kk[j * LM_T + r] = KEY_NONE;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < LM_QC / 2; ++u) {
      const int j = warp + 2 * u;
      if (j < nqc) {
#pragma unroll
        for (int g = 0; g < LM_T; g += 32) best[u] = warp_merge_smallest32(best[u], kk[j * LM_T + g + lane]);
      }
    }
  }
#pragma unroll
  for (int u = 0; u < LM_QC / 2; ++u) {
    const int j = warp + 2 * u;
    if (j < nqc && lane < k) out_pk[(int64_t)pairs[pbase + j] * k + lane] = best[u];
  }
}

// A warp per query: the k smallest of its nprobe x k per-list keys, sorted;
// tail 1e38 / -1, IP un-negated.
__global__ void __launch_bounds__(128)
    k_lm_merge(const uint64_t* __restrict__ out_pk, int64_t nq, int P, int k, bool ip,
               float* __restrict__ out_d, int64_t* __restrict__ out_l) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * 4 + warp;
  if (row >= nq) return;
  const uint64_t* src = out_pk + row * (int64_t)P * k;
  const int n = P * k;
  uint64_t best = KEY_NONE;
  for (int i0 = 0; i0 < n; i0 += 32)
    best = warp_merge_smallest32(best, i0 + lane < n ? src[i0 + lane] : KEY_NONE);
  if (lane < k) {
    float dd = 1e38f;
    int64_t ll = -1;
    if (best != KEY_NONE) {
      dd = key_dist(best);
      if (ip) dd = -dd;
      ll = (int64_t)key_id(best);
    }
    out_d[row * k + lane] = dd;
    out_l[row * k + lane] = ll;
  }
}

}  // namespace

void launch_ivfflat_scan(const float* q, int64_t nq, int d, int metric, const int32_t* probes,
                         int nprobe, int nlist, const int64_t* list_off, const float* rows,
                         const uint32_t* ids, int k, float* out_d, int64_t* out_l, cudaStream_t s) {
  if (nq == 0) return;
  MV_REQUIRE(nq <= 0x7fffffffll, MV_ERR_UNSUPPORTED, "too many queries in one batch");
  // rows per tile: as many as fit next to the query and the top-k buffer
  const size_t keys = (size_t)BlockTopK::smem_keys(k, TOP_BUF) * 8;
  const size_t budget = 200 * 1024;
  MV_REQUIRE(keys + (size_t)d * 4 + (size_t)32 * (d + 1) * 4 + 16 <= budget, MV_ERR_UNSUPPORTED,
             "IVF-Flat scan: d or k too large");
  int tr = (int)std::min<size_t>(FT, (budget - keys - (size_t)d * 4 - 16) / ((size_t)(d + 1) * 4));
  tr = std::max(32, tr / 32 * 32);
  const size_t smem = (((size_t)(d + (size_t)tr * (d + 1)) * 4 + 15) & ~size_t(15)) + keys;
  if (metric == MV_METRIC_L2) {
    smem_limit(k_ivfflat_scan<false>, smem);
    k_ivfflat_scan<false><<<(unsigned)nq, FT, smem, s>>>(q, d, probes, nprobe, nlist, list_off,
                                                        rows, ids, tr, k, out_d, out_l);
  } else {
    smem_limit(k_ivfflat_scan<true>, smem);
    k_ivfflat_scan<true><<<(unsigned)nq, FT, smem, s>>>(q, d, probes, nprobe, nlist, list_off, rows,
                                                       ids, tr, k, out_d, out_l);
  }
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}


size_t ivfflat_lm_scratch_bytes(int64_t nq, int nprobe, int nlist, int k) {
  const int64_t npairs = nq * nprobe;
  auto a = [](size_t b) { return (b + 255) & ~size_t(255); };
  return a((size_t)(nlist + 1) * 4) * 3 + a((size_t)(nlist + 1) * 8) + a((size_t)npairs * 4) +
         a((size_t)npairs * k * 8);
}

bool ivfflat_lm_supported(int64_t nq, int d, int nprobe, int k) {
  const size_t smem = (((size_t)(LM_QC * d + (size_t)LM_T * (d + 1)) * 4 + 15) & ~size_t(15)) +
                      (size_t)LM_QC * LM_T * 8;
  return k >= 1 && k <= 32 && nq * (int64_t)nprobe < (1ll << 31) && smem <= 200 * 1024;
}

void launch_ivfflat_scan_lm(const float* q, int64_t nq, int d, int metric, const int32_t* probes,
                            int nprobe, int nlist, const int64_t* list_off, const float* rows,
                            const uint32_t* ids, int k, float* out_d, int64_t* out_l, void* scratch,
                            cudaStream_t s) {
  if (nq == 0) return;
  MV_REQUIRE(ivfflat_lm_supported(nq, d, nprobe, k), MV_ERR_INTERNAL, "list-major IVF-Flat scan: unsupported shape");
  const int64_t npairs = nq * nprobe;
  auto a = [](size_t b) { return (b + 255) & ~size_t(255); };
  unsigned char* p = static_cast<unsigned char*>(scratch);
  int* cnt = reinterpret_cast<int*>(p);
  p += a((size_t)(nlist + 1) * 4);
  int* cursor = reinterpret_cast<int*>(p);
  p += a((size_t)(nlist + 1) * 4);
  int* istart = reinterpret_cast<int*>(p);
  p += a((size_t)(nlist + 1) * 4);
  int64_t* start = reinterpret_cast<int64_t*>(p);
  p += a((size_t)(nlist + 1) * 8);
  int32_t* pairs = reinterpret_cast<int32_t*>(p);
  p += a((size_t)npairs * 4);
  uint64_t* out_pk = reinterpret_cast<uint64_t*>(p);
  MV_CHECK_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (nlist + 1), s));
  MV_CHECK_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int) * (nlist + 1), s));
  MV_CHECK_CUDA(cudaMemsetAsync(out_pk, 0xff, sizeof(uint64_t) * npairs * k, s));
  const unsigned gp = (unsigned)((npairs + 255) / 256);
  k_lm_count<<<gp, 256, 0, s>>>(probes, npairs, nlist, cnt);
  k_lm_offsets<<<1, 1024, 0, s>>>(cnt, nlist, LM_QC, start, istart);
  k_lm_place<<<gp, 256, 0, s>>>(probes, npairs, nlist, start, cursor, pairs);
  count_launch();
  count_launch();
  count_launch();
  const size_t smem = (((size_t)(LM_QC * d + (size_t)LM_T * (d + 1)) * 4 + 15) & ~size_t(15)) +
                      (size_t)LM_QC * LM_T * 8;
  const unsigned items = (unsigned)((npairs + LM_QC - 1) / LM_QC + nlist);  // >= the work items
  if (metric == MV_METRIC_L2) {
    smem_limit(k_lm_scan<false>, smem);
    k_lm_scan<false><<<items, LM_T, smem, s>>>(q, d, nprobe, list_off, rows, ids, cnt, start,
                                                 istart, nlist, pairs, k, out_pk);
  } else {
    smem_limit(k_lm_scan<true>, smem);
    k_lm_scan<true><<<items, LM_T, smem, s>>>(q, d, nprobe, list_off, rows, ids, cnt, start, istart,
                                                nlist, pairs, k, out_pk);
  }
  count_launch();
  k_lm_merge<<<(unsigned)((nq + 3) / 4), 128, 0, s>>>(out_pk, nq, nprobe, k, metric != MV_METRIC_L2,
                                                      out_d, out_l);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
