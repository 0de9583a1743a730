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
#include <cuda_fp16.h>

#include <type_traits>

#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_fast.h"
#include "mv_select.cuh"
#include "mv_adc.cuh"

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
                  int32_t* __restrict__ probes, float* __restrict__ term, int* __restrict__ err) {
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
    const bool in_range = c < m && key_id(keys[c]) < (uint32_t)nlist;
    if (c < m && !in_range && lane == 0) atomicExch(err, 102);
    if (in_range) {
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

// Coarse step from the fused GEMM's per-segment candidates: the nc
// smallest of the ncand approximate keys, their exact FP32 distances, the
// nprobe smallest sorted ascending by (distance, list). Padding keys are made
// distinct (KEY_NONE - i) and never selected ahead of real ones.
__global__ void __launch_bounds__(FT)
    k_coarse_from_keys(const uint64_t* __restrict__ cand, int ncand, const float* __restrict__ q,
                       int d, const float* __restrict__ cent, int nlist, int metric, int nc,
                       int ncp, int nprobe, int32_t* __restrict__ probes, float* __restrict__ term,
                       int* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char smraw[];
  uint64_t* keys = reinterpret_cast<uint64_t*>(smraw);  // ncand
  uint64_t* sel = keys + ncand;                         // ncp
  float* qv = reinterpret_cast<float*>(sel + ncp);
  __shared__ RadixScratch rs;
  const int64_t row = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t pad0 = KEY_NONE - (uint64_t)ncand;
  for (int j = threadIdx.x; j < d; j += FT) qv[j] = q[row * d + j];
  for (int j = threadIdx.x; j < ncand; j += FT) {
    const uint64_t k = cand[row * ncand + j];
    keys[j] = k == KEY_NONE ? KEY_NONE - (uint64_t)j : k;
  }
  __syncthreads();
  const int r = block_radix_select<FT>(keys, ncand, nc, sel, rs);
  for (int j = threadIdx.x; j < r; j += FT) keys[j] = sel[j];
  __syncthreads();
  for (int c = warp; c < ncp; c += FT / 32) {
    uint64_t out = KEY_NONE - (uint64_t)c;
    const bool real = c < r && keys[c] <= pad0;
    const bool in_range = real && key_id(keys[c]) < (uint32_t)nlist;
    if (real && !in_range && lane == 0) atomicExch(err, 101);
    if (in_range) {
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
    const uint64_t key = sel[p];
    const bool ok = key < KEY_NONE - (uint64_t)ncp;
    probes[row * nprobe + p] = ok ? (int32_t)key_id(key) : -1;
    term[row * nprobe + p] = ok ? key_dist(key) : 0.0f;
  }
}

// Coarse step from the approximate distance matrix, one warp per query
// (nc <= 64). Each lane keeps its two smallest (distance, list) keys; the
// nc-th smallest of those 64 keys is a threshold T with at least nc keys of
// the row at or below it, usually a few dozen. Those are gathered, the nc
// smallest kept (the same set a top-nc heap keeps), their exact FP32
// distances computed as in k_coarse_from_keys, and the nprobe smallest
// written sorted by (distance, list). When more than CR_CAP keys sit at or
// below T, the exact nc-th smallest key is found by bisection over the key
// values first.
constexpr int CR_WARPS = 8, CR_CAP = 256;

__device__ __forceinline__ void warp_bitonic_sort(uint64_t* a, int n) {
  const int lane = threadIdx.x & 31;
  for (int k = 2; k <= n; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < n; i += 32) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const uint64_t x = a[i], y = a[ixj];
          const bool up = (i & k) == 0;
          if ((x > y) == up) {
            a[i] = y;
            a[ixj] = x;
          }
        }
      }
      __syncwarp();
    }
}

// B[0..nc): a query's nc smallest approximate (distance, list) keys, sorted
// (KEY_NONE where the row has fewer). Their exact FP32 distances (as
// k_coarse_from_keys) are sorted and the nprobe smallest written.
__device__ void coarse_recheck_warp(uint64_t* B, int64_t row, const float* __restrict__ q, int d,
                                    const float* __restrict__ cent, int nlist, int metric, int nc,
                                    int nprobe, int32_t* __restrict__ probes,
                                    float* __restrict__ term, int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const float* qr = q + row * d;
  const int ncp = next_pow2(nc);
  // CU candidates per round, so their row loads overlap; each distance is
  // computed exactly as in k_coarse_from_keys (lane-strided FMAs, xor tree).
  constexpr int CU = 8;
  for (int c0 = 0; c0 < ncp; c0 += CU) {
    uint32_t list[CU];
    bool ok[CU];
    float acc[CU];
#pragma unroll
    for (int u = 0; u < CU; ++u) {
      const int c = c0 + u;
      const uint64_t key = c < nc ? B[c] : KEY_NONE;
      list[u] = key_id(key);
      ok[u] = key != KEY_NONE && list[u] < (uint32_t)nlist;
      if (key != KEY_NONE && !ok[u] && lane == 0) atomicExch(err, 106);
      acc[u] = 0.0f;
    }
    if (d <= 128) {
      // every element of the round loaded before any is summed (one load
      // latency per round); the sums run in the same order as below
      float qv[4], cv[CU][4];
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        const int j = lane + 32 * jj;
        qv[jj] = j < d ? qr[j] : 0.0f;
#pragma unroll
        for (int u = 0; u < CU; ++u) cv[u][jj] = ok[u] && j < d ? cent[(int64_t)list[u] * d + j] : 0.0f;
      }
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        if (lane + 32 * jj >= d) break;
#pragma unroll
        for (int u = 0; u < CU; ++u) {
          if (metric == MV_METRIC_L2) {
            const float df = qv[jj] - cv[u][jj];
            acc[u] = fmaf(df, df, acc[u]);
          } else {
            acc[u] = fmaf(qv[jj], cv[u][jj], acc[u]);
          }
        }
      }
    } else {
      for (int j = lane; j < d; j += 32) {
        const float qj = qr[j];
#pragma unroll
        for (int u = 0; u < CU; ++u) {
          if (!ok[u]) continue;
          const float v = cent[(int64_t)list[u] * d + j];
          if (metric == MV_METRIC_L2) {
            const float df = qj - v;
            acc[u] = fmaf(df, df, acc[u]);
          } else {
            acc[u] = fmaf(qj, v, acc[u]);
          }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < CU; ++u)
      for (int o = 16; o > 0; o >>= 1) acc[u] += __shfl_xor_sync(0xffffffffu, acc[u], o);
    __syncwarp();
    if (lane == 0) {
#pragma unroll
      for (int u = 0; u < CU; ++u) {
        const int c = c0 + u;
        if (c < ncp)
          B[c] = ok[u] ? make_key(metric == MV_METRIC_L2 ? acc[u] : -acc[u], list[u])
                       : KEY_NONE - (uint64_t)c;
      }
    }
    __syncwarp();
  }
  warp_bitonic_sort(B, ncp);
  for (int p = lane; p < nprobe; p += 32) {
    const uint64_t key = B[p];
    const bool ok = key < KEY_NONE - (uint64_t)ncp;
    probes[row * nprobe + p] = ok ? (int32_t)key_id(key) : -1;
    term[row * nprobe + p] = ok ? key_dist(key) : 0.0f;
  }
}

__global__ void __launch_bounds__(CR_WARPS * 32)
    k_coarse_rows(const float* __restrict__ approx, int64_t nq, int nlist, const float* __restrict__ q,
                  int d, const float* __restrict__ cent, int metric, int nc, int nprobe,
                  int32_t* __restrict__ probes, float* __restrict__ term, int* __restrict__ err) {
  __shared__ uint64_t bufs[CR_WARPS][CR_CAP];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * CR_WARPS + warp;
  if (row >= nq) return;  // warps are independent: no block-wide barrier below
  uint64_t* B = bufs[warp];
  const float* arow = approx + row * (int64_t)nlist;
  // 1. the two smallest keys of each lane
  uint64_t m0 = KEY_NONE, m1 = KEY_NONE;
  for (int i = lane; i < nlist; i += 32) {
    const uint64_t k = make_key(arow[i], (uint32_t)i);
    if (k < m1) {
      if (k < m0) {
        m1 = m0;
        m0 = k;
      } else {
        m1 = k;
      }
    }
  }
  B[lane] = m0;
  B[32 + lane] = m1;
  __syncwarp();
  warp_bitonic_sort(B, 64);
  const uint64_t T = B[nc - 1];  // nc <= min(nlist, 64) keys are valid
  __syncwarp();
  // 2. gather the keys <= T
  auto gather = [&](uint64_t thr) -> int {
    int cnt = 0;
    for (int i0 = 0; i0 < nlist; i0 += 32) {
      const int i = i0 + lane;
      const uint64_t k = i < nlist ? make_key(arow[i], (uint32_t)i) : KEY_NONE;
      const bool pass = i < nlist && k <= thr;
      const unsigned bal = __ballot_sync(0xffffffffu, pass);
      const int pos = cnt + __popc(bal & ((1u << lane) - 1u));
      if (pass && pos < CR_CAP) B[pos] = k;
      cnt += __popc(bal);
    }
    return cnt;
  };
  int cnt = gather(T);
  if (cnt > CR_CAP) {
    // bisection: the smallest key value with at least nc keys at or below it
    uint64_t lo = 0, hi = T;
    while (lo < hi) {
      const uint64_t mid = lo + ((hi - lo) >> 1);
      int c = 0;
      for (int i = lane; i < nlist; i += 32) c += make_key(arow[i], (uint32_t)i) <= mid ? 1 : 0;
      for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
      if (c >= nc) hi = mid;
      else lo = mid + 1;
    }
    __syncwarp();
    cnt = gather(lo);  // exactly nc keys (keys are distinct)
  }
  __syncwarp();
  int np2 = 32;
  while (np2 < cnt) np2 <<= 1;
  for (int i = cnt + lane; i < np2; i += 32) B[i] = KEY_NONE;
  __syncwarp();
  warp_bitonic_sort(B, np2);
  coarse_recheck_warp(B, row, q, d, cent, nlist, metric, nc, nprobe, probes, term, err);
}

// The row's candidate keys (segment lists concatenated) sorted in registers;
// the nc <= 32 smallest end up in v[0] of lanes 0 .. nc - 1.
template <int RR>
__device__ __forceinline__ uint64_t coarse_lists_smallest(const uint64_t* __restrict__ lists,
                                                          int64_t row, int nseg, int cap, int n,
                                                          int o1, int o2, int o3) {
  const int lane = threadIdx.x & 31;
  uint64_t v[RR];
#pragma unroll
  for (int r = 0; r < RR; ++r) {
    const int i = (r << 5) | lane;
    uint64_t key = KEY_NONE;
    if (i < n) {
      const int sg = (i >= o1) + (i >= o2) + (i >= o3);
      const int base = sg == 0 ? 0 : sg == 1 ? o1 : sg == 2 ? o2 : o3;
      key = lists[((int64_t)row * nseg + sg) * cap + (i - base)];
    }
    v[r] = key;
  }
  warp_sort_regs<RR>(v);
  return v[0];
}

// Per-row lists of the two-pass coarse GEMM -> the row's nc smallest keys,
// sorted, in out[row * ncp + j] (KEY_NONE past nc or past the row's keys),
// one warp per row.
__global__ void __launch_bounds__(CR_WARPS * 32)
    k_lists_smallest(const uint64_t* __restrict__ lists, const int* __restrict__ counts, int nseg,
                     int cap, int64_t nq, int nc, int ncp, uint64_t* __restrict__ out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * CR_WARPS + warp;
  if (row >= nq) return;
  const int c = lane < nseg ? min(max(counts[row * nseg + lane], 0), cap) : 0;
  int incl = c;
#pragma unroll
  for (int o = 1; o < 4; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  const int o1 = __shfl_sync(0xffffffffu, incl, 0);
  const int o2 = nseg > 1 ? __shfl_sync(0xffffffffu, incl, 1) : 1 << 30;
  const int o3 = nseg > 2 ? __shfl_sync(0xffffffffu, incl, 2) : 1 << 30;
  const int n = __shfl_sync(0xffffffffu, incl, nseg - 1);
  const int p1 = nseg > 1 ? o1 : 1 << 30;
  uint64_t best;
  if (n <= 32) best = coarse_lists_smallest<1>(lists, row, nseg, cap, n, p1, o2, o3);
  else if (n <= 64) best = coarse_lists_smallest<2>(lists, row, nseg, cap, n, p1, o2, o3);
  else if (n <= 128) best = coarse_lists_smallest<4>(lists, row, nseg, cap, n, p1, o2, o3);
  else best = coarse_lists_smallest<8>(lists, row, nseg, cap, n, p1, o2, o3);
  if (lane < ncp) out[row * ncp + lane] = lane < nc ? best : KEY_NONE;
}

// Per-row lists of the two-pass coarse GEMM -> the nc smallest keys, their
// exact FP32 distances and the nprobe nearest lists, one warp per query (the
// same selection and recheck as k_coarse_rows; nseg <= 4, nseg * cap <= 256,
// nc <= 32).
__global__ void __launch_bounds__(CR_WARPS * 32)
    k_coarse_lists(const uint64_t* __restrict__ lists, const int* __restrict__ counts, int nseg,
                   int cap, int64_t nq, int nlist, const float* __restrict__ q, int d,
                   const float* __restrict__ cent, int metric, int nc, int nprobe,
                   int32_t* __restrict__ probes, float* __restrict__ term, int* __restrict__ err) {
  __shared__ uint64_t bufs[CR_WARPS][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * CR_WARPS + warp;
  if (row >= nq) return;  // warps are independent: no block-wide barrier below
  const int c = lane < nseg ? min(max(counts[row * nseg + lane], 0), cap) : 0;
  int incl = c;  // inclusive prefix over the (at most 4) segments
#pragma unroll
  for (int o = 1; o < 4; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  const int o1 = __shfl_sync(0xffffffffu, incl, 0);
  const int o2 = nseg > 1 ? __shfl_sync(0xffffffffu, incl, 1) : 1 << 30;
  const int o3 = nseg > 2 ? __shfl_sync(0xffffffffu, incl, 2) : 1 << 30;
  const int n = __shfl_sync(0xffffffffu, incl, nseg - 1);
  const int p1 = nseg > 1 ? o1 : 1 << 30;
  uint64_t best;
  if (n <= 32) best = coarse_lists_smallest<1>(lists, row, nseg, cap, n, p1, o2, o3);
  else if (n <= 64) best = coarse_lists_smallest<2>(lists, row, nseg, cap, n, p1, o2, o3);
  else if (n <= 128) best = coarse_lists_smallest<4>(lists, row, nseg, cap, n, p1, o2, o3);
  else best = coarse_lists_smallest<8>(lists, row, nseg, cap, n, p1, o2, o3);
  uint64_t* B = bufs[warp];
  B[lane] = best;
  __syncwarp();
  coarse_recheck_warp(B, row, q, d, cent, nlist, metric, nc, nprobe, probes, term, err);
}

// ---------------------------------------------------------------------------
// Bank-rotated tables. A warp that looks up one subspace's 256-entry table
// for 32 candidates at once sends 32 random codes to random banks (about 3.5
// wavefronts per lookup instruction, more with repeats). Here every
// subspace's table lives in one bank per copy: in a pass of S subspaces
// (S = 8, 16 or 32) with C = 32 / S copies, entry (m, c) of subspace
// m = p S + j sits at word (c + 256 p) * 32 + j + S h for copy h. Lane l
// (r = l mod S, h = l / S) looks up subspace (r + s) mod S at step s, in copy
// h, so the 32 lanes of a step read 32 different banks whatever the codes:
// one wavefront per lookup instruction. Each lane rotates its candidate's
// code bytes by r first (a word barrel shift and a funnel shift), so step s
// reads byte s of the rotated code. Subspaces past M (M not a multiple of S)
// are zero tables read with zero code bytes.
//
// Entries are integers: the query's table values times 2^e, rounded, with e
// chosen from a Cauchy-Schwarz bound (sum over m of ||q_m|| times the
// largest codeword norm of m) so that every sum stays below 2^30. Integer
// sums do not depend on the order of the terms, so a candidate's distance
// does not depend on the lane (the rotation) that computes it.
// ---------------------------------------------------------------------------
template <int WS>
__device__ __forceinline__ void load_code_words(const uint8_t* __restrict__ row, int M, int p,
                                                uint32_t (&w)[WS]) {
  const int nw = M >> 2, w0 = p * WS;
  if ((M & 15) == 0 && (WS & 3) == 0) {
#pragma unroll
    for (int i = 0; i < WS; i += 4) {
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (w0 + i < nw) v = *reinterpret_cast<const uint4*>(row + 4 * (w0 + i));
      w[i] = v.x;
      w[i + 1] = v.y;
      w[i + 2] = v.z;
      w[i + 3] = v.w;
    }
  } else if ((M & 7) == 0 && (WS & 1) == 0) {
#pragma unroll
    for (int i = 0; i < WS; i += 2) {
      uint2 v = make_uint2(0u, 0u);
      if (w0 + i < nw) v = *reinterpret_cast<const uint2*>(row + 4 * (w0 + i));
      w[i] = v.x;
      w[i + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < WS; ++i)
      w[i] = w0 + i < nw ? *reinterpret_cast<const uint32_t*>(row + 4 * (w0 + i)) : 0u;
  }
}

// Per-lane state of the rotated lookups.
template <int S>
struct RotLane {
  static constexpr int WS = S / 4;
  int boff[S];  // byte offset, within a 128-byte table row, of step s's bank
  int qw, rb8;  // word rotation and bit shift of the lane's code bytes
  __device__ __forceinline__ void init(int lane) {
    const int r = lane & (S - 1), h = lane / S;
#pragma unroll
    for (int s = 0; s < S; ++s) boff[s] = 4 * (((r + s) & (S - 1)) + S * h);
    qw = r >> 2;
    rb8 = 8 * (r & 3);
  }
  // Sum of the table entries of one pass of a code (words w, zero past M).
  __device__ __forceinline__ int sum(const int* tab, const uint32_t (&w)[WS]) const {
    uint32_t L[WS];
#pragma unroll
    for (int i = 0; i < WS; ++i) L[i] = w[i];
#pragma unroll
    for (int b = 1; b < WS; b <<= 1) {
      const bool f = (qw & b) != 0;
      uint32_t T[WS];
#pragma unroll
      for (int i = 0; i < WS; ++i) T[i] = f ? L[(i + b) % WS] : L[i];
#pragma unroll
      for (int i = 0; i < WS; ++i) L[i] = T[i];
    }
    uint32_t o[WS];
#pragma unroll
    for (int i = 0; i < WS; ++i) o[i] = __funnelshift_r(L[i], L[(i + 1) % WS], rb8);
    const char* tb = reinterpret_cast<const char*>(tab);
    int a0 = 0, a1 = 0;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const uint32_t c = (o[s >> 2] >> (8 * (s & 3))) & 255u;
      const int v = *reinterpret_cast<const int*>(tb + (c << 7) + boff[s]);
      if (s & 1) a1 += v;
      else a0 += v;
    }
    return a0 + a1;
  }
};

// The query's integer tables in the rotated layout: entry (m, c) =
// rint(mul * <q_m, C[m][c]>), with mul = table scale * 2^e (and the FP16
// codebook's power-of-two scale when pq16 is used). Lane l computes
// subspace p S + (l mod S) for code j C + l / S and the C lanes of a slot
// swap values so each writes all C codes of the group into its own bank.
template <int NT, int S>
__device__ __forceinline__ void build_rot_tables(int* tab, const float* qv, const float* pq,
                                                 const __half* pq16, int M, int dsub, float mul) {
  constexpr int C = 32 / S;
  constexpr int GROUPS = 256 / C;
  constexpr int NW = NT / 32;
  constexpr int U = 4;  // codeword loads in flight per lane
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = lane & (S - 1), h = lane / S;
  const int P = (M + S - 1) / S;
  const int total = P * GROUPS;
  auto store = [&](int it, int vi) {
    const int p = it / GROUPS, j = it - p * GROUPS;
#pragma unroll
    for (int hh = 0; hh < C; ++hh) {
      const int vv = C == 1 ? vi : __shfl_sync(0xffffffffu, vi, slot + S * hh);
      tab[((j * C + hh) + 256 * p) * 32 + lane] = vv;
    }
  };
  if (pq16 && (dsub == 8 || dsub == 4)) {
    // Work item it = (pass p, group j): this lane's entry (m, c) with
    // m = p S + slot, c = j C + h. U items per lane are loaded, then used.
    for (int it0 = warp; it0 < total; it0 += NW * U) {
      uint4 cw[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int it = it0 + u * NW;
        const int p = it / GROUPS, j = it - p * GROUPS;
        const int m = p * S + slot, c = j * C + h;
        cw[u] = make_uint4(0u, 0u, 0u, 0u);
        if (it < total && m < M) {
          if (dsub == 8) {
            cw[u] = __ldg(reinterpret_cast<const uint4*>(pq16 + ((int64_t)m * 256 + c) * 8));
          } else {
            const uint2 v = __ldg(reinterpret_cast<const uint2*>(pq16 + ((int64_t)m * 256 + c) * 4));
            cw[u].x = v.x;
            cw[u].y = v.y;
          }
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int it = it0 + u * NW;
        if (it >= total) break;  // warp-uniform
        const int m = (it / GROUPS) * S + slot;
        int vi = 0;
        if (m < M) {
          const float* xm = qv + m * dsub;
          const float4 qa = *reinterpret_cast<const float4*>(xm);
          const float2 c0 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].x));
          const float2 c1 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].y));
          float dot = qa.x * c0.x;
          dot = fmaf(qa.y, c0.y, dot);
          dot = fmaf(qa.z, c1.x, dot);
          dot = fmaf(qa.w, c1.y, dot);
          if (dsub == 8) {
            const float4 qb = *reinterpret_cast<const float4*>(xm + 4);
            const float2 c2 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].z));
            const float2 c3 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].w));
            dot = fmaf(qb.x, c2.x, dot);
            dot = fmaf(qb.y, c2.y, dot);
            dot = fmaf(qb.z, c3.x, dot);
            dot = fmaf(qb.w, c3.y, dot);
          }
          vi = __float2int_rn(dot * mul);
        }
        store(it, vi);
      }
    }
  } else {
    for (int it = warp; it < total; it += NW) {
      const int p = it / GROUPS, j = it - p * GROUPS;
      const int m = p * S + slot, c = j * C + h;
      int vi = 0;
      if (m < M) {
        const float* xm = qv + m * dsub;
        const float* cp = pq + ((int64_t)m * 256 + c) * dsub;
        float dot = 0.0f;
        for (int t = 0; t < dsub; ++t) dot = fmaf(xm[t], __ldg(cp + t), dot);
        vi = __float2int_rn(dot * mul);
      }
      store(it, vi);
    }
  }
}

// ADC scan, one CTA per query. The probed lists are laid end to end in one
// candidate index space (prefix sums of their lengths in shared memory), so
// every thread has work whatever the list lengths. Candidate keys are staged
// as (ordered distance, CSR position) word pairs; whenever the next chunk
// would overflow the staging area, and once at the end, a radix select keeps
// the R smallest. The shortlist is written unsorted (the rerank orders it),
// or sorted when it is the final answer.
// MODE 0: FP32 tables, 1: FP16 tables, 8 / 16 / 32: bank-rotated integer
// tables with S = MODE subspaces per pass.
template <int NT, int MODE>
__global__ void __launch_bounds__(NT, 1024 / NT) k_ivfpq_scan_fast(FastScanArgs a) {
  constexpr int FT = NT;
  constexpr bool HALF = MODE == 1;
  constexpr int S = MODE >= 8 ? MODE : 8;  // rotated modes only
  constexpr bool ROT = MODE >= 8;
  using LutT = typename std::conditional<HALF, __half, float>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int M = a.M, d = a.d, dsub = d / M;
  const int tab_words = ROT ? ((M + S - 1) / S) * 256 * 32 : M * 256;
  // The table region is sized for 4-byte entries in every mode.
  LutT* lut = reinterpret_cast<LutT*>(smraw);
  int* tab = reinterpret_cast<int*>(smraw);
  float* qv = reinterpret_cast<float*>(smraw) + tab_words;
  uint64_t* outb =
      reinterpret_cast<uint64_t*>(smraw + (((size_t)(tab_words + d) * 4 + 15) & ~size_t(15)));
  uint32_t* khi = reinterpret_cast<uint32_t*>(outb + a.Rp);
  uint32_t* klo = khi + a.cap;
  int64_t* poff = reinterpret_cast<int64_t*>(klo + a.cap);  // nprobe list offsets
  int* pbeg = reinterpret_cast<int*>(poff + a.nprobe);      // nprobe + 1 prefix sums
  float* pterm = reinterpret_cast<float*>(pbeg + a.nprobe + 1);
  __shared__ RadixScratch rs;
  __shared__ int s_fill;
  __shared__ int s_q;
  __shared__ unsigned s_amax;  // FP16 tables: largest |entry| (float bits)
  __shared__ unsigned long long s_kth;  // the R-th smallest key of the last select
  __shared__ int s_e;          // rotated tables: entries are in units of 2^-s_e
  __shared__ int s_bad;        // rotated tables: non-finite query or codebook bound
  const int lane = threadIdx.x & 31;
  // One query per CTA, or (with a.counter) a persistent CTA that takes
  // queries from a global counter in a.order until none are left.
  for (int iter = 0;; ++iter) {
  int qi;
  if (a.counter) {
    __syncthreads();  // the previous query is done with shared memory
    if (threadIdx.x == 0) s_q = atomicAdd(a.counter, 1);
    __syncthreads();
    qi = s_q;
    if (qi >= a.nq) break;
  } else {
    if (iter > 0) break;
    qi = blockIdx.x;
  }
  const int64_t row = a.order ? a.order[qi] : qi;
  const int nprobe = a.nprobe_q ? min(max(a.nprobe_q[row], 1), a.nprobe) : a.nprobe;
  if (threadIdx.x == 0) s_fill = 0;
  for (int j = threadIdx.x; j < d; j += FT) qv[j] = a.q[row * d + j];
  // probe table: offsets, lengths -> prefix sums (warp 0)
  if (threadIdx.x < 32) {
    int carry = 0;
    for (int p0 = 0; p0 < nprobe; p0 += 32) {
      const int p = p0 + lane;
      int len = 0;
      if (p < nprobe) {
        int list = a.probes[row * a.nprobe + p];
        if (list >= a.nlist) {
          atomicExch(a.err, 103);
          list = -1;
        }
        int64_t off = 0;
        if (list >= 0) {
          off = a.list_off[list];
          len = (int)(a.list_off[list + 1] - off);
        }
        poff[p] = off;
        pterm[p] = a.term[row * a.nprobe + p];
      }
      int incl = len;
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      if (p < nprobe) pbeg[p] = carry + incl - len;
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (lane == 0) pbeg[nprobe] = carry;
  }
  __syncthreads();
  const float scale = a.metric == MV_METRIC_L2 ? -2.0f : -1.0f;
  // FP16 tables carry a per-query power-of-two scale so no entry overflows
  // (a first pass finds the largest magnitude); sums stay in FP32.
  float lscale = 1.0f;
  if constexpr (ROT) {
    // e from sum_m ||q_m|| * max_c ||C[m][c]|| (with slack for the FP16
    // codebook's rounding and the FP32 dot products): |sum| < 2^30.
    if (threadIdx.x < 32) {
      float b = 0.0f;
      for (int m = lane; m < M; m += 32) {
        float s2 = 0.0f;
        for (int t = 0; t < dsub; ++t) s2 = fmaf(qv[m * dsub + t], qv[m * dsub + t], s2);
        b += sqrtf(s2) * a.pq_cn[m];
      }
      for (int o = 16; o > 0; o >>= 1) b += __shfl_xor_sync(0xffffffffu, b, o);
      if (lane == 0) {
        b *= fabsf(scale) * 1.0625f;
        const bool bad = !(b <= 3.0e38f);  // NaN or infinite
        int e = 0;
        if (!bad && b > 0.0f) e = min(max(29 - (ilogbf(b) + 1), -120), 120);
        s_e = e;
        s_bad = bad ? 1 : 0;
      }
    }
    __syncthreads();
    const float mul = scale * (a.pq16 ? a.pq16_inv : 1.0f) * __int_as_float((s_e + 127) << 23);
    build_rot_tables<NT, S>(tab, qv, a.pq, a.pq16, M, dsub, mul);
    lscale = __int_as_float((127 - s_e) << 23);  // 2^-e
  } else if constexpr (HALF) {
    if (threadIdx.x == 0) s_amax = 0u;
    __syncthreads();
    float mx = 0.0f;
    if (a.pq16) build_lut16<NT>([&](int, float v) { mx = fmaxf(mx, fabsf(v)); }, qv, a.pq16, M, dsub, scale * a.pq16_inv);
    else build_lut<NT>([&](int, float v) { mx = fmaxf(mx, fabsf(v)); }, qv, a.pq, M, dsub, scale);
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) atomicMax(&s_amax, __float_as_uint(mx));
    __syncthreads();
    const float amax = __uint_as_float(s_amax);
    if (amax > 0.0f) lscale = exp2f((float)(ilogbf(amax) - 14));  // amax / lscale < 2^15
    const float inv = 1.0f / lscale;  // a power of two: exact
    if (a.pq16)
      build_lut16<NT>([&](int i, float v) { lut[i] = __float2half_rn(v * inv); }, qv, a.pq16, M,
                      dsub, scale * a.pq16_inv);
    else
      build_lut<NT>([&](int i, float v) { lut[i] = __float2half_rn(v * inv); }, qv, a.pq, M, dsub,
                    scale);
  } else {
    if (a.pq16) build_lut16<NT>([&](int i, float v) { lut[i] = v; }, qv, a.pq16, M, dsub, scale * a.pq16_inv);
    else build_lut<NT>([&](int i, float v) { lut[i] = v; }, qv, a.pq, M, dsub, scale);
  }
  __syncthreads();
  RotLane<S> rl;  // set up after the tables so its registers are not live during the build
  if constexpr (ROT) rl.init(lane);
  const int total = pbeg[nprobe];
  const int chunk = a.cap - a.R;
  int m = 0;
  // Per-thread probe cursors of the thread's first and second candidates
  // (each one's indices only grow), with the probe's end, CSR base (offset
  // - first index) and term kept in registers.
  int p = 0, pend = pbeg[1];
  int64_t pbase = poff[0];  // pbeg[0] = 0
  float pt = pterm[0];
  int p1 = 0, pend1 = pend;
  int64_t pbase1 = pbase;
  float pt1 = pt;
  // Keys at or above `bound` cannot enter the shortlist once R keys below
  // it have been seen; it tightens after every intermediate select.
  unsigned long long bound = ~0ull;
  for (int base = 0; base < total; base += chunk) {
    const int len = min(chunk, total - base);
    if (m + len > a.cap) {
      const int r = block_hist_select<FT>(khi, klo, m, a.R, outb, rs, &s_kth);
      for (int j = threadIdx.x; j < r; j += FT) {
        const uint64_t k = outb[j];
        khi[j] = (uint32_t)(k >> 32);
        klo[j] = (uint32_t)k;
      }
      if (r == a.R) bound = s_kth;  // the R-th smallest key so far
      m = r;
      if (threadIdx.x == 0) s_fill = m;
      __syncthreads();
    }
    // Two candidates per thread per step: both rows' loads are issued before
    // either table walk.
    for (int j0 = 0; j0 < len; j0 += 2 * FT) {
      const int j = j0 + threadIdx.x;
      const bool has0 = j < len;
      const bool has1 = j + FT < len;
      const int c0 = base + j, c1 = c0 + FT;
      // Lanes without a candidate keep their cursor and use position 0 (a
      // valid entry: the index is not empty), so no load leaves the lists.
      if (has0 && c0 >= pend) {  // c0 < pbeg[nprobe]: p stops below nprobe
        do {
          ++p;
        } while (pbeg[p + 1] <= c0);
        pend = pbeg[p + 1];
        pbase = poff[p] - pbeg[p];
        pt = pterm[p];
      }
      int64_t pos0c = has0 ? pbase + c0 : 0;
      const float t0 = has0 ? pt : 0.0f;
      if (has1 && c1 >= pend1) {
        do {
          ++p1;
        } while (pbeg[p1 + 1] <= c1);
        pend1 = pbeg[p1 + 1];
        pbase1 = poff[p1] - pbeg[p1];
        pt1 = pterm[p1];
      }
      int64_t pos1 = has1 ? pbase1 + c1 : 0;
      const float t1 = has1 ? pt1 : 0.0f;
      bool keep0 = has0, keep1 = has1;
      if ((has0 && (pos0c < 0 || pos0c >= a.ntotal)) || (has1 && (pos1 < 0 || pos1 >= a.ntotal))) {
        atomicExch(a.err, 104);  // never expected: skip both, stay warp-uniform
        pos0c = 0;
        pos1 = 0;
        keep0 = keep1 = false;
      }
      if (a.filter) {  // filtered ids never enter the shortlist
        const uint32_t id0 = a.ids[pos0c], id1 = a.ids[pos1];
        if ((int64_t)id0 < a.filter_len && a.filter[id0] != 0) keep0 = false;
        if ((int64_t)id1 < a.filter_len && a.filter[id1] != 0) keep1 = false;
      }
      const float v0 = a.vterm ? a.vterm[pos0c] : 0.0f;
      const float v1 = a.vterm ? a.vterm[pos1] : 0.0f;
      float d0, d1;
      if constexpr (ROT) {
        constexpr int WS = S / 4;
        const int P = (M + S - 1) / S;
        int s0 = 0, s1 = 0;
        for (int pp = 0; pp < P; ++pp) {
          uint32_t w0[WS], w1[WS];
          load_code_words<WS>(a.codes + pos0c * M, M, pp, w0);
          load_code_words<WS>(a.codes + pos1 * M, M, pp, w1);
          s0 += rl.sum(tab + pp * 256 * 32, w0);
          s1 += rl.sum(tab + pp * 256 * 32, w1);
        }
        d0 = fmaf((float)s0, lscale, t0 + v0);
        d1 = fmaf((float)s1, lscale, t1 + v1);
        if (s_bad) d0 = d1 = __int_as_float(0x7fc00000);
      } else if constexpr (HALF) {
        d0 = fmaf(lscale, adc_fast(lut, a.codes + pos0c * M, M, 0.0f), t0 + v0);
        d1 = fmaf(lscale, adc_fast(lut, a.codes + pos1 * M, M, 0.0f), t1 + v1);
      } else {
        d0 = adc_fast(lut, a.codes + pos0c * M, M, t0 + v0);
        d1 = adc_fast(lut, a.codes + pos1 * M, M, t1 + v1);
      }
      const unsigned long long k0 = ((unsigned long long)float_to_ordered(d0) << 32) | (uint32_t)pos0c;
      const unsigned long long k1 = ((unsigned long long)float_to_ordered(d1) << 32) | (uint32_t)pos1;
      const bool in0 = keep0 && k0 < bound;
      const bool in1 = keep1 && k1 < bound;
      const unsigned b0 = __ballot_sync(0xffffffffu, in0);
      const unsigned b1 = __ballot_sync(0xffffffffu, in1);
      int wbase = 0;
      if (lane == 0 && (b0 | b1)) wbase = atomicAdd(&s_fill, __popc(b0) + __popc(b1));
      wbase = __shfl_sync(0xffffffffu, wbase, 0);
      const unsigned below = (1u << lane) - 1u;
      if (in0) {
        const int slot = wbase + __popc(b0 & below);
        khi[slot] = (uint32_t)(k0 >> 32);
        klo[slot] = (uint32_t)k0;
      }
      if (in1) {
        const int slot = wbase + __popc(b0) + __popc(b1 & below);
        khi[slot] = (uint32_t)(k1 >> 32);
        klo[slot] = (uint32_t)k1;
      }
    }
    __syncthreads();
    m = s_fill;
    __syncthreads();
  }
  const int r = block_hist_select<FT>(khi, klo, m, a.R, outb, rs, &s_kth);
  if (a.sorted) {
    for (int j = r + threadIdx.x; j < a.Rp; j += FT) outb[j] = KEY_NONE;
    __syncthreads();
    block_bitonic_sort(outb, a.Rp);
  }
  for (int i = threadIdx.x; i < a.R; i += FT) a.out_keys[row * a.R + i] = i < r ? outb[i] : KEY_NONE;
  }  // queries
}

// FP32 distances of U shortlisted rows (positions pos, 0xffffffff = none)
// to the query qv, accumulated per lane in acc: float4 loads of the lane's
// 4-element slices (scalar elements when d is not a multiple of 4). The
// warp's sum of acc (xor tree) is the distance; every exact rerank path
// uses this arithmetic.
template <int U>
__device__ __forceinline__ void rerank_rows_fp32(const RerankArgs& a, const float* qv,
                                                 const uint32_t* pos, float* acc) {
  const int d = a.d;
  const int lane = threadIdx.x & 31;
  if ((d & 3) == 0) {
    for (int j = lane * 4; j < d; j += 128) {
      float4 v[U];
#pragma unroll
      for (int u = 0; u < U; ++u)
        v[u] = pos[u] != 0xffffffffu ? *reinterpret_cast<const float4*>(a.raw + (int64_t)pos[u] * d + j)
                                     : make_float4(0.f, 0.f, 0.f, 0.f);
      const float q0 = qv[j], q1 = qv[j + 1], q2 = qv[j + 2], q3 = qv[j + 3];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (a.metric == MV_METRIC_L2) {
          const float d0 = q0 - v[u].x, d1 = q1 - v[u].y, d2 = q2 - v[u].z, d3 = q3 - v[u].w;
          acc[u] = fmaf(d0, d0, fmaf(d1, d1, fmaf(d2, d2, fmaf(d3, d3, acc[u]))));
        } else {
          acc[u] = fmaf(q0, v[u].x, fmaf(q1, v[u].y, fmaf(q2, v[u].z, fmaf(q3, v[u].w, acc[u]))));
        }
      }
    }
  } else {
    for (int j = lane; j < d; j += 32) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (pos[u] == 0xffffffffu) continue;
        const float x = a.raw[(int64_t)pos[u] * d + j];
        if (a.metric == MV_METRIC_L2) {
          const float df = qv[j] - x;
          acc[u] = fmaf(df, df, acc[u]);
        } else {
          acc[u] = fmaf(qv[j], x, acc[u]);
        }
      }
    }
  }
}

// Results of one query from its k smallest keys outb[0, k) (sorted;
// padding keys above KEY_NONE - R become unfilled slots).
__device__ __forceinline__ void rerank_write(const RerankArgs& a, int64_t row, const uint64_t* outb,
                                             int t0, int nt) {
  const int kq = a.k_q ? min(max(a.k_q[row], 0), a.k) : a.k;
  for (int i = t0; i < a.k; i += nt) {
    const uint64_t key = outb[i];
    float dd = a.fill_d;
    int64_t ll = -1;
    if (i < kq && key < KEY_NONE - (uint64_t)a.R) {
      dd = key_dist(key);
      if (a.metric != MV_METRIC_L2) dd = -dd;
      ll = (int64_t)key_id(key);
    }
    a.out_d[row * a.k + i] = dd;
    a.out_l[row * a.k + i] = ll;
  }
}

// Exact FP32 rerank of the shortlist against the raw rows (CSR order), one
// CTA per query: a warp per candidate row (float4 loads, U rows in flight per
// warp; keys and ids of a warp's 32 candidates loaded once, a lane each),
// then the k smallest (distance, id) keys, sorted.
__global__ void __launch_bounds__(FT) k_rerank_fast(RerankArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int d = a.d;
  float* qv = reinterpret_cast<float*>(smraw);
  uint64_t* ck = reinterpret_cast<uint64_t*>(smraw + (((size_t)d * 4 + 15) & ~size_t(15)));
  uint64_t* outb = ck + a.R;     // kp (power of two >= k)
  uint64_t* part = outb + a.kp;  // FT keys (k <= 32 selection)
  __shared__ RadixScratch rs;
  const int64_t row = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int j = threadIdx.x; j < d; j += FT) qv[j] = a.q[row * d + j];
  __syncthreads();
  const uint64_t* cand = a.cand + row * a.R;
  constexpr int U = 8;
  for (int c0 = warp * 32; c0 < a.R; c0 += FT) {
    uint32_t mpos = 0xffffffffu, mid = 0;
    if (c0 + lane < a.R) {
      const uint64_t key = cand[c0 + lane];
      if (key != KEY_NONE) {
        mpos = key_id(key);
        if ((int64_t)mpos >= a.ntotal) {
          atomicExch(a.err, 105);
          mpos = 0xffffffffu;
        } else {
          mid = a.ids ? a.ids[mpos] : mpos;
        }
      }
    }
    const int nloc = min(32, a.R - c0);
    for (int u0 = 0; u0 < nloc; u0 += U) {
      uint32_t pos[U];
      float acc[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint32_t p = __shfl_sync(0xffffffffu, mpos, (u0 + u) & 31);
        pos[u] = u0 + u < nloc ? p : 0xffffffffu;
        acc[u] = 0.0f;
      }
      rerank_rows_fp32<U>(a, qv, pos, acc);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        float t = acc[u];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        const uint32_t id = __shfl_sync(0xffffffffu, mid, (u0 + u) & 31);
        const int c = c0 + u0 + u;
        if (lane == 0 && u0 + u < nloc) {
          ck[c] = pos[u] == 0xffffffffu
                      ? KEY_NONE - (uint64_t)c  // distinct keys for empty slots
                      : make_key(a.metric == MV_METRIC_L2 ? t : -t, id);
        }
      }
    }
  }
  __syncthreads();
  if (a.k <= 32) {
    // The k smallest keys: every warp keeps the 32 smallest of its share in
    // registers, warp 0 merges the warps' sets (keys are distinct, so this
    // is the same set as a radix select).
    uint64_t best = KEY_NONE;
    for (int c0 = warp * 32; c0 < a.R; c0 += FT)
      best = warp_merge_smallest32(best, c0 + lane < a.R ? ck[c0 + lane] : KEY_NONE);
    part[warp * 32 + lane] = best;
    __syncthreads();
    if (warp == 0) {
      best = part[lane];
      for (int w = 1; w < FT / 32; ++w) best = warp_merge_smallest32(best, part[w * 32 + lane]);
      if (lane < a.kp) outb[lane] = best;
    }
    __syncthreads();
  } else {
    const int r = block_radix_select<FT>(ck, a.R, a.k, outb, rs);
    for (int j = r + threadIdx.x; j < a.kp; j += FT) outb[j] = KEY_NONE;
    __syncthreads();
    block_bitonic_sort(outb, a.kp);
  }
  rerank_write(a, row, outb, threadIdx.x, FT);
}

// Certified rerank (k <= 32), one warp per query. Every shortlisted row's
// distance is first computed from its 8-bit copy (a quarter of the FP32
// bytes, one 128-byte line per row at d = 128) and turned into an interval
// that provably holds the FP32 distance the exact pass computes. With y8 the
// row the copy decodes to (y8_j = fmaf(S_j, 1 + u_j 2^-15, a''_j), the FP32
// expression the copy was made with) and r >= ||y - y8||: the prescreen
// value's own summation error, the triangle inequality with r (L2; widened
// by the rounding of the per-query constants its one-FMA differences use)
// or Cauchy-Schwarz with ||q|| and ||y8|| (IP), and the exact pass's
// summation error (both bounded by gamma = (d + 64) * 2^-24 relative to the
// sum of |terms|), with 2^-20 of slack for the bound arithmetic. The k-th
// smallest upper end of any k or more candidates bounds the query's k-th
// smallest key; a candidate whose lower end exceeds it has k candidates
// strictly closer and is dropped. The survivors are computed in FP32 with
// k_rerank_fast's arithmetic, so the results are the ones the full FP32
// pass gives.
//
// The 8-bit rows are gathered RC_ROWS at a time into a two-round ring in
// shared memory with asynchronous 16-byte copies: round i + 2's copies are
// issued as soon as round i is decoded, so every warp keeps two rounds of
// row bytes in flight. Decoding reads one 4-byte word of every row per lane
// (bank-conflict free), and a transposing butterfly gives each lane a row's
// sum.
__host__ __device__ constexpr size_t rerank_cert_warp_bytes(int d, int R, int RC_ROWS) {
  // query | 2 x 32 rows of d8 bytes | survivors' keys (R) | lower ends |
  // positions | upper ends / survivor list
  return ((((size_t)d * 4 + 15) & ~size_t(15)) + 2 * RC_ROWS * (size_t)(((d + 15) & ~15)) +
          (size_t)R * 20 + 15) & ~size_t(15);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// RC_ROWS rows per round (32, or 16 with half the accumulators, registers
// and ring for more warps per SM).
template <int RC_ROWS>
__global__ void __launch_bounds__(128, RC_ROWS == 32 ? 4 : 6) k_rerank_cert(RerankArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int d = a.d, d8 = a.d8;
  const int nwarps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * nwarps + warp;
  if (row >= a.nq) return;  // warps are independent: no block-wide barrier below
  const size_t qbytes = ((size_t)d * 4 + 15) & ~size_t(15);
  unsigned char* base = smraw + (size_t)warp * rerank_cert_warp_bytes(d, a.R, RC_ROWS);
  float* qv = reinterpret_cast<float*>(base);
  unsigned char* ring = base + qbytes;                       // 2 x RC_ROWS rows of d8 bytes
  const size_t rbytes = (size_t)RC_ROWS * d8;
  uint64_t* sk = reinterpret_cast<uint64_t*>(ring + 2 * rbytes);  // R: survivors' keys
  float* blo = reinterpret_cast<float*>(sk + a.R);                // R lower ends
  uint32_t* spos = reinterpret_cast<uint32_t*>(blo + a.R);        // R positions
  uint32_t* bhi = spos + a.R;                                     // R upper ends (ordered)
  int* slist = reinterpret_cast<int*>(bhi);                       // R survivors (after bhi)
  const float INF = __int_as_float(0x7f800000);
  const float gam = (float)(d + 64) * 5.9604645e-08f;  // (d + 64) * 2^-24
  const float up = 1.0f + 9.5367432e-07f, dn = 1.0f - 9.5367432e-07f;  // 1 +- 2^-20
  for (int j = lane; j < d; j += 32) qv[j] = a.q[row * d + j];
  const uint64_t* cand = a.cand + row * a.R;
  constexpr int KU = 8;  // shortlist keys in flight per lane
  for (int c0 = 0; c0 < a.R; c0 += 32 * KU) {
    uint64_t kk[KU];
#pragma unroll
    for (int u = 0; u < KU; ++u) {
      const int c = c0 + u * 32 + lane;
      kk[u] = c < a.R ? __ldg(cand + c) : KEY_NONE;
    }
#pragma unroll
    for (int u = 0; u < KU; ++u) {
      const int c = c0 + u * 32 + lane;
      uint32_t mpos = 0xffffffffu;
      if (kk[u] != KEY_NONE) {
        mpos = key_id(kk[u]);
        if ((int64_t)mpos >= a.ntotal) {
          atomicExch(a.err, 105);
          mpos = 0xffffffffu;
        }
      }
      if (c < a.R) spos[c] = mpos;
    }
  }
  __syncwarp();
  const int nrounds = (a.R + RC_ROWS - 1) / RC_ROWS;
  const int chunks = d8 >> 4;  // 16-byte pieces per row
  const bool pow2c = (chunks & (chunks - 1)) == 0;
  const int csh = 31 - __clz(chunks);
  // issue round t's row copies into ring slot t & 1 (empty slots copy nothing)
  auto issue = [&](int t) {
    if (t < nrounds) {
      const uint32_t dst0 = (uint32_t)__cvta_generic_to_shared(ring + (size_t)(t & 1) * rbytes);
      if (chunks == 8) {  // 128-byte rows: the lane copies piece lane % 8 of rows lane / 8 + 4 i
        const int ch = lane & 7;
#pragma unroll
        for (int i = 0; i < RC_ROWS / 4; ++i) {
          const int u = (lane >> 3) + 4 * i;
          const int c = t * RC_ROWS + u;
          const uint32_t p = c < a.R ? spos[c] : 0xffffffffu;
          if (p != 0xffffffffu)
            cp_async16(dst0 + (uint32_t)(u * 128 + ch * 16), a.raw8 + (int64_t)p * 128 + ch * 16);
        }
      } else {
        for (int e = lane; e < RC_ROWS * chunks; e += 32) {
          // (row, piece) of copy e: shifts when the piece count is a power of two
          const int u = pow2c ? e >> csh : e / chunks, ch = e - u * chunks;
          const int c = t * RC_ROWS + u;
          const uint32_t p = c < a.R ? spos[c] : 0xffffffffu;
          if (p != 0xffffffffu)
            cp_async16(dst0 + (uint32_t)(u * d8 + ch * 16), a.raw8 + (int64_t)p * d8 + ch * 16);
        }
      }
    }
    cp_async_commit();  // one group per round, empty or not
  };
  issue(0);
  issue(1);
  const bool l2 = a.metric == MV_METRIC_L2;
  float qn = 0.0f;  // IP: upper bound on ||q||
  float eq = 0.0f;  // L2: upper bound on ||t||, t_j = (q_j - a''_j) - fl(q_j - a''_j)
  if (!l2) {
    for (int j = lane; j < d; j += 32) qn = fmaf(qv[j], qv[j], qn);
    for (int o = 16; o > 0; o >>= 1) qn += __shfl_xor_sync(0xffffffffu, qn, o);
    qn = sqrtf(qn * (1.0f + 2.0f * gam)) * up;
  } else {
    for (int j = lane; j < d; j += 32) {
      const float x = qv[j], b = -a.dim8[j].x;
      const float sm = x + b, bp = sm - x;
      const float t = (x - (sm - bp)) + (b - bp);  // two-sum: x + b - sm exactly
      eq = fmaf(t, t, eq);
    }
    for (int o = 16; o > 0; o >>= 1) eq += __shfl_xor_sync(0xffffffffu, eq, o);
    eq = sqrtf(eq * (1.0f + 2.0f * gam)) * up;
  }
  // Element constants of the lane's first 128 elements. L2 computes each
  // difference in one rounding as fma(-S, V, c) with c = fl(q - a''), which
  // is (q - y8) + eta, |eta_j| <= |t_j| + 2^-24 |y8_j| (y8_j = fl(S V + a''),
  // one rounding): the bound below widens r by eq + 2^-24 ||y8||. IP decodes
  // y8 = fma(S, V, a''). Elements past d decode to 0 against a query
  // element of 0 (byte 0 gives V = 1).
  float q0[4], k0[4], m0[4];  // query; L2: (c, -S), IP: (a'', S)
#pragma unroll
  for (int tt = 0; tt < 4; ++tt) {
    const int j = lane * 4 + tt;
    const bool in = j < d;
    const float2 ds = in ? a.dim8[j] : make_float2(-1.0f, 1.0f);
    q0[tt] = in ? qv[j] : 0.0f;
    k0[tt] = l2 ? q0[tt] - ds.x : ds.x;
    m0[tt] = l2 ? -ds.y : ds.y;
  }
  for (int t = 0; t < nrounds; ++t) {
    const int c0 = t * RC_ROWS;
    const int c = c0 + (lane & (RC_ROWS - 1));
    const uint32_t mine = c < a.R ? spos[c] : 0xffffffffu;
    const float2 meta = mine != 0xffffffffu ? __ldg(a.rmeta + mine) : make_float2(0.0f, 0.0f);
    cp_async_wait<1>();  // round t's group has landed (round t + 1's may be in flight)
    __syncwarp();
    const unsigned char* buf = ring + (size_t)(t & 1) * rbytes;
    float acc[RC_ROWS];
#pragma unroll
    for (int u = 0; u < RC_ROWS; ++u) acc[u] = 0.0f;
    // lane: elements j .. j + 3 of every row (one 4-byte word)
    for (int j0 = 0; j0 < d; j0 += 128) {
      const int j = j0 + lane * 4;
      const bool jin = j < d;
      float qj[4], kj[4], mj[4];
#pragma unroll
      for (int tt = 0; tt < 4; ++tt) {
        if (j0 == 0) {  // the first 128 elements' constants stay in registers
          qj[tt] = q0[tt];
          kj[tt] = k0[tt];
          mj[tt] = m0[tt];
        } else {
          const bool in = j + tt < d;
          const float2 ds = in ? a.dim8[j + tt] : make_float2(-1.0f, 1.0f);
          qj[tt] = in ? qv[j + tt] : 0.0f;
          kj[tt] = l2 ? qj[tt] - ds.x : ds.x;
          mj[tt] = l2 ? -ds.y : ds.y;
        }
      }
      const unsigned char* rowp = buf + j;
#pragma unroll
      for (int u = 0; u < RC_ROWS; ++u, rowp += d8) {
        const uint32_t w = jin ? *reinterpret_cast<const uint32_t*>(rowp) : 0u;
        float e[4];  // L2: c - S V; IP: y8
#pragma unroll
        for (int tt = 0; tt < 4; ++tt)
          e[tt] = fmaf(mj[tt], __uint_as_float(__byte_perm(w, 0x3F800000u, 0x7604u + 16u * tt)), kj[tt]);
        if (l2) {
          acc[u] = fmaf(e[0], e[0], fmaf(e[1], e[1], fmaf(e[2], e[2], fmaf(e[3], e[3], acc[u]))));
        } else {
          acc[u] = fmaf(qj[0], e[0], fmaf(qj[1], e[1], fmaf(qj[2], e[2], fmaf(qj[3], e[3], acc[u]))));
        }
      }
    }
    __syncwarp();  // every lane has read the slot before it is refilled
    issue(t + 2);
    // transposing butterfly: lane l ends with row c0 + (l mod RC_ROWS)'s sum
    // (with 16 rows, lanes l and l + 16 add their halves at the end)
#pragma unroll
    for (int w = RC_ROWS / 2; w >= 1; w >>= 1) {
      const bool upper = (lane & w) != 0;
#pragma unroll
      for (int i = 0; i < w; ++i) {
        const float send = upper ? acc[i] : acc[i + w];
        const float keep = upper ? acc[i + w] : acc[i];
        acc[i] = keep + __shfl_xor_sync(0xffffffffu, send, w);
      }
    }
    if constexpr (RC_ROWS == 16) acc[0] += __shfl_xor_sync(0xffffffffu, acc[0], 16);
    if (lane < RC_ROWS && c < a.R) {
      float lo = INF, hi = INF;  // empty slots never survive
      if (mine != 0xffffffffu) {
        const float tv = acc[0];
        const float r = meta.x, yn = meta.y;
        if (!(fabsf(tv) < INF) || !(r < INF) || !(yn < INF) || !(eq < INF)) {  // computed exactly
          lo = -INF;
          hi = INF;
        } else if (l2) {
          const float rr = (r + eq + yn * 5.9604645e-08f) * up;  // r + ||eta||
          const float slo = sqrtf(tv * (1.0f - 2.0f * gam)) * dn - rr * up;
          const float shi = sqrtf(tv * (1.0f + 2.0f * gam)) * up + rr * up;
          const float m = fmaxf(slo, 0.0f);
          lo = m * m * (1.0f - 2.0f * gam) * dn;
          hi = shi * shi * (1.0f + 2.0f * gam) * up;
        } else {
          const float e = qn * (gam * yn + r + gam * (yn + r)) * up;
          lo = (-tv - e) * (-tv - e < 0.0f ? up : dn);
          hi = (-tv + e) * (-tv + e < 0.0f ? dn : up);
        }
      }
      blo[c] = lo;
      bhi[c] = float_to_ordered(hi);
    }
  }
  cp_async_wait<0>();
  __syncwarp();
  // The bound: the k-th smallest upper end of a subset of the shortlist (k
  // distinct candidates have upper ends at or below it, so it bounds the
  // k-th smallest key; k <= 32). The subset is each lane's two smallest
  // upper ends (64 values): it holds the whole shortlist's k smallest unless
  // one lane holds three of them. Bounding by each group of 32's own k-th
  // smallest instead leaves several times more survivors, as a query's k
  // nearest rows spread over the groups.
  uint32_t m1 = 0xffffffffu, m2 = 0xffffffffu;  // (ordered INF is below 0xffffffff)
  for (int c = lane; c < a.R; c += 32) {
    const uint32_t x = bhi[c];
    m2 = min(m2, max(m1, x));
    m1 = min(m1, x);
  }
  const uint32_t hk = warp_kth_smallest64(m1, m2, a.k);
  __syncwarp();  // bhi is read by every lane before slist overwrites it
  const float hkf = hk == 0xffffffffu ? INF : ordered_to_float(hk);
  int ns = 0;
  for (int c0 = 0; c0 < a.R; c0 += 32) {
    const int c = c0 + lane;
    const bool keep = c < a.R && blo[c] <= hkf;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) slist[ns + __popc(m & ((1u << lane) - 1u))] = c;
    ns += __popc(m);
  }
  __syncwarp();
  // exact FP32 keys of the survivors (k_rerank_fast's arithmetic)
  constexpr int U = 8;
  for (int i0 = 0; i0 < ns; i0 += U) {
    uint32_t pos[U];
    float acc[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      pos[u] = i0 + u < ns ? spos[slist[i0 + u]] : 0xffffffffu;
      acc[u] = 0.0f;
    }
    // the survivors' ids: lane u of the group loads survivor u's beside the rows
    uint32_t myid = 0;
    {
      const uint32_t pp = lane < U && i0 + lane < ns ? spos[slist[i0 + lane]] : 0xffffffffu;
      if (pp != 0xffffffffu) myid = a.ids ? a.ids[pp] : pp;
    }
    rerank_rows_fp32<U>(a, qv, pos, acc);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      float tv = acc[u];
      for (int o = 16; o > 0; o >>= 1) tv += __shfl_xor_sync(0xffffffffu, tv, o);
      const uint32_t id = __shfl_sync(0xffffffffu, myid, u);
      if (lane == 0 && i0 + u < ns) {
        const int c = slist[i0 + u];
        sk[i0 + u] = pos[u] == 0xffffffffu ? KEY_NONE - (uint64_t)c
                                           : make_key(a.metric == MV_METRIC_L2 ? tv : -tv, id);
      }
    }
  }
  __syncwarp();
  // the k smallest keys are the survivors' smallest (every other key is
  // padding, above all real keys)
  uint64_t best = KEY_NONE;
  for (int i0 = 0; i0 < ns; i0 += 32)
    best = warp_merge_smallest32(best, i0 + lane < ns ? sk[i0 + lane] : KEY_NONE);
  uint64_t* outb = sk;  // reuse: 32 sorted keys
  __syncwarp();
  outb[lane] = best;
  __syncwarp();
  rerank_write(a, row, outb, lane, 32);
}

// Per-dimension minimum and maximum of the rows (ordered words, combined
// with atomics into dimord[0, d) and dimord[d, 2d)); a block walks a range
// of rows with one thread per dimension.
__global__ void k_dim_minmax(const float* __restrict__ raw, int64_t n, int d, int64_t rows_per_block,
                             uint32_t* __restrict__ dimord) {
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_block;
  const int64_t r1 = min(n, r0 + rows_per_block);
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    uint32_t lo = 0xffffffffu, hi = 0u;
    for (int64_t r = r0; r < r1; ++r) {
      const uint32_t o = float_to_ordered(raw[r * d + j]);
      lo = min(lo, o);
      hi = max(hi, o);
    }
    if (r0 < r1) {
      atomicMin(&dimord[j], lo);
      atomicMax(&dimord[d + j], hi);
    }
  }
}

__global__ void k_dim_init(uint32_t* dimord, int d) {
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    dimord[j] = 0xffffffffu;
    dimord[d + j] = 0u;
  }
}

// Per dimension (a''_j, S_j) of the 8-bit copy: s_j a power of two and
// a_j = floor(min_j / s_j) s_j with 255 s_j >= max_j - a_j (s_j = 1 for a
// constant or non-finite dimension), stored as S_j = 2^15 s_j and
// a''_j = a_j - S_j, so that y8 = fmaf(S_j, V, a''_j) decodes code u from
// the float V = 1 + u 2^-15, whose bits are 0x3F800000 | (u << 8) (one
// byte permute). a''_j is exact while |a_j / s_j| < 2^24 - 2^15; every row
// bound is computed from the decoded values, so the copy stays certified
// either way.
__global__ void k_dim_steps(const uint32_t* __restrict__ dimord, int d, float2* __restrict__ dim8) {
  for (int j = threadIdx.x; j < d; j += blockDim.x) {
    const float lo = ordered_to_float(dimord[j]), hi = ordered_to_float(dimord[d + j]);
    float s = 1.0f, a = 0.0f;
    if (isfinite(lo) && isfinite(hi)) {
      const float range = hi - lo;
      if (range > 0.0f && range < __int_as_float(0x7f800000)) {
        s = ldexpf(1.0f, ilogbf(range) - 7);
        if (255.0f * s < range) s *= 2.0f;
        if (hi - floorf(lo / s) * s > 255.0f * s) s *= 2.0f;
      }
      a = floorf(lo / s) * s;
    }
    dim8[j] = make_float2(a - 32768.0f * s, 32768.0f * s);
  }
}

// 8-bit copy of each row, an upper bound on ||y - y8|| and on ||y8||, one
// warp per row. The squared sums carry a relative error of at most
// (d + 2) 2^-24 (non-negative terms), covered by the (d + 64) 2^-23
// inflation, and 2^-21 more covers the square root.
__global__ void k_rerank_rows8(const float* __restrict__ raw, int64_t n, int d, int d8,
                               const float2* __restrict__ dim8, uint8_t* __restrict__ raw8,
                               float2* __restrict__ rmeta) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= n) return;
  float e2 = 0.0f, y2 = 0.0f;
  bool finite = true;
  for (int j = lane; j < d8; j += 32) {
    uint32_t code = 0;
    if (j < d) {
      const float y = raw[r * d + j];
      const float2 as = dim8[j];
      const float a = as.x + as.y;               // a_j (exact when a''_j is)
      const float st = as.y * 3.0517578125e-05f;  // s_j = S_j 2^-15
      const float t = rintf((y - a) / st);
      code = (uint32_t)(int)fminf(fmaxf(t, 0.0f), 255.0f);  // NaN -> 0
      const float y8 = fmaf(as.y, __uint_as_float(0x3F800000u | (code << 8)), as.x);
      const float df = y - y8;
      finite = finite && isfinite(y) && isfinite(y8);
      e2 = fmaf(df, df, e2);
      y2 = fmaf(y8, y8, y2);
    }
    raw8[r * d8 + j] = (uint8_t)code;
  }
  for (int o = 16; o > 0; o >>= 1) {
    e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    y2 += __shfl_xor_sync(0xffffffffu, y2, o);
  }
  finite = __all_sync(0xffffffffu, finite);
  if (lane == 0) {
    const float INF = __int_as_float(0x7f800000);
    const float infl = 1.0f + (float)(d + 64) * 1.1920929e-07f;
    const float up = 1.0f + 4.7683716e-07f;  // 1 + 2^-21
    const float rr = sqrtf(e2 * infl) * up, yn = sqrtf(y2 * infl) * up;
    rmeta[r] = finite && rr < INF && yn < INF ? make_float2(rr, yn) : make_float2(INF, INF);
  }
}

// Shortlist without rerank: the first k keys (already sorted) -> results.
__global__ void k_short_to_results(const uint64_t* __restrict__ keys, int64_t nq, int R, int k,
                                   const uint32_t* __restrict__ ids, int metric,
                                   const int32_t* __restrict__ k_q, float* __restrict__ out_d,
                                   int64_t* __restrict__ out_l) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq * k) return;
  const int64_t r = i / k;
  const int j = (int)(i - r * k);
  const uint64_t key = keys[r * R + j];
  if (key == KEY_NONE || (k_q && j >= k_q[r])) {
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
                        float* term, int* err, cudaStream_t s) {
  if (nq == 0) return;
  const int ncp = next_pow2(nc);
  const size_t smem = (size_t)(CC_CHUNK + nc + ncp) * 8 + (size_t)d * 4;
  MV_REQUIRE(smem <= 200 * 1024, MV_ERR_UNSUPPORTED, "coarse select: nprobe or d too large");
  smem_attr(k_coarse_fast, smem);
  k_coarse_fast<<<(unsigned)nq, FT, smem, s>>>(approx, nlist, q, d, cent, metric, nc, ncp, nprobe,
                                                probes, term, err);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_coarse_rows(const float* approx, int64_t nq, int nlist, const float* q, int d,
                        const float* cent, int metric, int nc, int nprobe, int32_t* probes,
                        float* term, int* err, cudaStream_t s) {
  if (nq == 0) return;
  MV_REQUIRE(nc >= 1 && nc <= 64 && nc <= nlist && nprobe <= nc, MV_ERR_UNSUPPORTED,
             "coarse rows: nc must be in [nprobe, min(64, nlist)]");
  k_coarse_rows<<<(unsigned)((nq + CR_WARPS - 1) / CR_WARPS), CR_WARPS * 32, 0, s>>>(
      approx, nq, nlist, q, d, cent, metric, nc, nprobe, probes, term, err);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_lists_smallest(const uint64_t* lists, const int* counts, int nseg, int cap, int64_t nq,
                           int nc, uint64_t* out, cudaStream_t s) {
  if (nq == 0) return;
  MV_REQUIRE((int64_t)nseg * cap <= CR_CAP && nseg <= 4 && nc >= 1 && nc <= 32, MV_ERR_INTERNAL,
             "lists smallest: too many keys per row");
  k_lists_smallest<<<(unsigned)((nq + CR_WARPS - 1) / CR_WARPS), CR_WARPS * 32, 0, s>>>(
      lists, counts, nseg, cap, nq, nc, next_pow2(nc), out);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_coarse_lists(const uint64_t* lists, const int* counts, int nseg, int cap, int64_t nq,
                         int nlist, const float* q, int d, const float* cent, int metric, int nc,
                         int nprobe, int32_t* probes, float* term, int* err, cudaStream_t s) {
  if (nq == 0) return;
  MV_REQUIRE(nc >= 1 && nc <= 64 && nc <= nlist && nprobe <= nc, MV_ERR_UNSUPPORTED,
             "coarse lists: nc must be in [nprobe, min(64, nlist)]");
  MV_REQUIRE((int64_t)nseg * cap <= CR_CAP && nseg <= 4 && nc <= 32, MV_ERR_INTERNAL,
             "coarse lists: too many keys per row");
  k_coarse_lists<<<(unsigned)((nq + CR_WARPS - 1) / CR_WARPS), CR_WARPS * 32, 0, s>>>(
      lists, counts, nseg, cap, nq, nlist, q, d, cent, metric, nc, nprobe, probes, term, err);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_coarse_from_keys(const uint64_t* cand, int64_t nq, int ncand, const float* q, int d,
                             const float* cent, int nlist, int metric, int nc, int nprobe,
                             int32_t* probes, float* term, int* err, cudaStream_t s) {
  if (nq == 0) return;
  const int ncp = next_pow2(nc);
  const size_t smem = (size_t)(ncand + ncp) * 8 + (size_t)d * 4;
  MV_REQUIRE(smem <= 200 * 1024, MV_ERR_UNSUPPORTED, "coarse merge: too many candidates");
  smem_attr(k_coarse_from_keys, smem);
  k_coarse_from_keys<<<(unsigned)nq, FT, smem, s>>>(cand, ncand, q, d, cent, nlist, metric, nc, ncp,
                                                     nprobe, probes, term, err);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

int fast_scan_cap(int R) { return std::max(2048, 2 * R + 1024); }

// Pass width of the bank-rotated tables for M subspaces, 0 when the scan
// keeps the plain layout.
int fast_scan_rot(const FastScanArgs& a, int lut) {
  if (lut != 3 || !a.pq_cn || (a.M & 3) != 0 || a.M < 8) return 0;
  return a.M <= 8 ? 8 : (a.M <= 16 ? 16 : 32);
}

size_t fast_scan_smem(const FastScanArgs& a) {
  const size_t tab_words =
      a.rot ? (size_t)((a.M + a.rot - 1) / a.rot) * 256 * 32 : (size_t)a.M * 256;
  return (((size_t)(tab_words + a.d) * 4 + 15) & ~size_t(15)) + (size_t)next_pow2(a.R) * 8 +
         (size_t)fast_scan_cap(a.R) * 8 + (size_t)a.nprobe * 8 + (size_t)(a.nprobe + 1) * 4 +
         (size_t)a.nprobe * 4;
}

// Threads per CTA nt (128, 256 or 512); grid: one CTA per query, or with
// a.counter a persistent grid of `persistent_ctas` CTAs.
void launch_ivfpq_scan_fast(FastScanArgs a, cudaStream_t s, int nt, int persistent_ctas,
                            int lut) {
  if (a.nq == 0) return;
  // lut 6: the bank-rotated fixed-point table scan with per-candidate slots
  if (lut == 6 && ivfpq_rt_supported(a)) {
    launch_ivfpq_scan_rt(a, s, nt, persistent_ctas);
    return;
  }
  MV_REQUIRE(lut != 6, MV_ERR_UNSUPPORTED, "rotated-table scan: unsupported M, d or codebook");
  if (lut == 4 && launch_ivfpq_scan_staged(a, s, nt, persistent_ctas, a.stage_entries)) return;
  a.cap = fast_scan_cap(a.R);
  a.Rp = next_pow2(a.R);
  a.rot = fast_scan_rot(a, lut);
  const size_t smem = fast_scan_smem(a);
  MV_REQUIRE(smem <= 220 * 1024, MV_ERR_UNSUPPORTED, "fast IVF-PQ scan: M, d or shortlist too large");
  MV_REQUIRE(!a.counter || persistent_ctas > 0, MV_ERR_INTERNAL, "persistent scan without a grid");
  const unsigned grid = a.counter ? (unsigned)std::min<int64_t>(persistent_ctas, a.nq) : (unsigned)a.nq;
  auto go = [&](auto kernel, int threads) {
    smem_attr(kernel, smem);
    kernel<<<grid, threads, smem, s>>>(a);
  };
  auto pick = [&](auto mode) {
    constexpr int MODE = decltype(mode)::value;
    if (nt == 128) go(k_ivfpq_scan_fast<128, MODE>, 128);
    else if (nt == 512) go(k_ivfpq_scan_fast<512, MODE>, 512);
    else go(k_ivfpq_scan_fast<256, MODE>, 256);
  };
  if (a.rot == 8) pick(std::integral_constant<int, 8>());
  else if (a.rot == 16) pick(std::integral_constant<int, 16>());
  else if (a.rot == 32) pick(std::integral_constant<int, 32>());
  else if (lut == 1) pick(std::integral_constant<int, 1>());  // 0, 2 (and 4 unstaged): FP32
  else pick(std::integral_constant<int, 0>());
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_rerank_fast(RerankArgs a, cudaStream_t s) {
  if (a.nq == 0) return;
  a.kp = next_pow2(a.k);
  const size_t qbytes = ((size_t)a.d * 4 + 15) & ~size_t(15);
  // rows per round of the certified rerank: 16 (80 registers, six CTAs of
  // four warps per SM) measured 0.161 ms against 0.168 ms for 32 at the
  // 1M x 128 headline shape
  constexpr int kRows = 16;
  const size_t wbytes = rerank_cert_warp_bytes(a.d, a.R, kRows);
  const int cw = (int)std::min<size_t>(4, (96 * 1024) / wbytes);  // warps per CTA
  if (a.raw8 && a.rmeta && a.dim8 && a.d8 == rerank8_row_bytes(a.d) && a.k <= 32 && a.R >= 32 &&
      cw >= 1) {
    const size_t csmem = (size_t)cw * wbytes;
    smem_attr(k_rerank_cert<kRows>, csmem);
    k_rerank_cert<kRows><<<(unsigned)((a.nq + cw - 1) / cw), cw * 32, csmem, s>>>(a);
    count_launch();
    MV_CHECK_CUDA(cudaGetLastError());
    return;
  }
  const size_t smem = qbytes + (size_t)(a.R + a.kp + FT) * 8;
  MV_REQUIRE(smem <= 220 * 1024, MV_ERR_UNSUPPORTED, "rerank: d or shortlist too large");
  smem_attr(k_rerank_fast, smem);
  k_rerank_fast<<<(unsigned)a.nq, FT, smem, s>>>(a);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_rerank_rows8(const float* raw, int64_t n, int d, uint32_t* dimord, float2* dim8,
                         uint8_t* raw8, float2* rmeta, cudaStream_t s) {
  if (n == 0) return;
  const int d8 = rerank8_row_bytes(d);
  k_dim_init<<<1, 256, 0, s>>>(dimord, d);
  count_launch();
  const int64_t per = 256;
  k_dim_minmax<<<(unsigned)((n + per - 1) / per), 128, 0, s>>>(raw, n, d, per, dimord);
  count_launch();
  k_dim_steps<<<1, 256, 0, s>>>(dimord, d, dim8);
  count_launch();
  k_rerank_rows8<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(raw, n, d, d8, dim8, raw8, rmeta);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_short_to_results(const uint64_t* keys, int64_t nq, int R, int k, const uint32_t* ids,
                             int metric, float* out_d, int64_t* out_l, cudaStream_t s,
                             const int32_t* k_q) {
  const int64_t total = nq * k;
  if (total == 0) return;
  k_short_to_results<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(keys, nq, R, k, ids, metric,
                                                                     k_q, out_d, out_l);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
