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

}  // namespace mv
