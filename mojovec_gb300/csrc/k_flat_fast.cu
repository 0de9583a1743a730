// Fast form of the flat scan (index/index_flat.mojo:260-325 semantics for the
// result layout): the BF16 tensor-core GEMM with the per-row heap epilogue
// (k_umma.cu) leaves, per query and column segment, the K smallest
// (BF16 distance, row) keys. This file merges the segments into the query's
// shortlist of R keys and, without rerank, turns the first k into results.
//
// When a segment keeps fewer keys than the shortlist needs (K < R), a full
// segment whose largest kept key is below the shortlist's R-th key may have
// dropped a key that belongs in the shortlist; the query is then flagged
// and the host recomputes it with the exact FP32 scan. When K >= R that
// cannot happen: K keys below the R-th key of the union would make it at
// least the (R + 1)-th.
#include "mv_fast.h"
#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"

namespace mv {
namespace {

constexpr int MT = 256;

__global__ void __launch_bounds__(MT)
    k_flat_merge(const uint64_t* __restrict__ cand, int nseg, int ncp, int kseg, int R,
                 uint64_t* __restrict__ out_keys, int k, int Rp, const float* __restrict__ qnorm,
                 int metric, float fill_d, float* __restrict__ out_d, int64_t* __restrict__ out_l,
                 int* __restrict__ overflow) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ncand = nseg * ncp;
  uint64_t* keys = reinterpret_cast<uint64_t*>(smraw);  // ncand
  uint64_t* sel = keys + ncand;                         // Rp (power of two >= R)
  __shared__ RadixScratch rs;
  __shared__ unsigned long long s_thr;
  __shared__ int s_over;
  const int64_t row = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t* c = cand + row * (int64_t)ncand;
  for (int j = threadIdx.x; j < ncand; j += MT) {
    const uint64_t key = c[j];
    keys[j] = key == KEY_NONE ? KEY_NONE - (uint64_t)j : key;  // distinct padding
  }
  if (threadIdx.x == 0) s_over = 0;
  __syncthreads();
  const int r = block_radix_select<MT>(keys, ncand, R, sel, rs);
  // R-th smallest key of the union (the largest selected one)
  unsigned long long mx = 0ull;
  for (int j = threadIdx.x; j < r; j += MT) mx = sel[j] > mx ? sel[j] : mx;
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = t > mx ? t : mx;
  }
  if (threadIdx.x == 0) s_thr = 0ull;
  __syncthreads();
  if (lane == 0) atomicMax(&s_thr, mx);
  __syncthreads();
  if (kseg < R && overflow) {
    const uint64_t thr = s_thr;
    for (int sg = warp; sg < nseg; sg += MT / 32) {
      bool full = true;
      unsigned long long smax = 0ull;
      for (int j = lane; j < kseg; j += 32) {
        const uint64_t key = c[(int64_t)sg * ncp + j];
        full = full && key != KEY_NONE;
        smax = key > smax ? key : smax;
      }
      full = __all_sync(0xffffffffu, full);
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, smax, o);
        smax = t > smax ? t : smax;
      }
      if (lane == 0 && full && smax < thr) s_over = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) overflow[row] = s_over;
  }
  const uint64_t pad0 = KEY_NONE - (uint64_t)ncand;  // keys above it are padding
  if (out_keys) {
    for (int j = threadIdx.x; j < R; j += MT)
      out_keys[row * R + j] = (j < r && sel[j] <= pad0) ? sel[j] : KEY_NONE;
    return;
  }
  // No rerank: the k smallest, sorted, with the row's ||q||^2 added back.
  for (int j = r + threadIdx.x; j < Rp; j += MT) sel[j] = KEY_NONE;
  __syncthreads();
  block_bitonic_sort(sel, Rp);
  for (int i = threadIdx.x; i < k; i += MT) {
    const uint64_t key = i < r ? sel[i] : KEY_NONE;
    float dd = fill_d;
    int64_t ll = -1;
    if (key <= pad0) {
      const float kd = key_dist(key);
      dd = metric == MV_METRIC_L2 ? fmaxf(kd + qnorm[row], 0.0f) : -kd;
      ll = (int64_t)key_id(key);
    }
    out_d[row * k + i] = dd;
    out_l[row * k + i] = ll;
  }
}

// SQ8 on the tensor cores: the GEMM kept, per output segment, the K
// largest e (e = 2 q.x - ||x||^2 for L2, e = q.x for IP; exact integers),
// keyed (-e, row). Here each candidate gets the reference's distance
// (index_flat_sq8.mojo:526-583 via quantization/sq8.mojo:62-79): L2
// Float32(max(||q||^2 + ||x||^2 - 2 q.x, 0)) * scale^2, IP -Float32(q.x) *
// scale^2, and the canonical key (distance, row); the R smallest are the
// shortlist. Rounding can give equal distances to different e, so a row a
// segment dropped (e <= its smallest kept e) could tie into the shortlist;
// the query is flagged whenever a full segment's smallest kept e maps to a
// distance not above the shortlist's largest, and the host then scans it.
// The shortlist is written sorted ascending.
__device__ __forceinline__ float sq8_dist_from_e(float e, uint32_t qn, bool ip, float scale_sq) {
  if (ip) return __fmul_rn(-e, scale_sq);  // e = q.x exactly, -Float32(q.x) * scale^2
  const int64_t dd = (int64_t)qn - (int64_t)e;  // ||q||^2 + ||x||^2 - 2 q.x
  const uint32_t u = (uint32_t)(dd > 0 ? dd : 0);
  return __fmul_rn(__uint2float_rn(u), scale_sq);
}

__global__ void __launch_bounds__(MT)
    k_sq8_merge(const uint64_t* __restrict__ cand, int nseg, int ncp, int kseg, int R,
                const uint32_t* __restrict__ qnorm, int ip, float scale_sq,
                uint64_t* __restrict__ out_keys, int* __restrict__ flag) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ncand = nseg * ncp;
  uint64_t* keys = reinterpret_cast<uint64_t*>(smraw);  // ncand
  uint64_t* sel = keys + ncand;                         // Rp = next_pow2(R)
  const int Rp = next_pow2(R);
  __shared__ RadixScratch rs;
  __shared__ unsigned long long s_thr;
  __shared__ int s_flag;
  const int64_t row = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t* c = cand + row * (int64_t)ncand;
  const uint32_t qn = qnorm[row];
  for (int j = threadIdx.x; j < ncand; j += MT) {
    const uint64_t key = c[j];
    uint64_t ck = KEY_NONE - (uint64_t)j;  // distinct padding
    if (key != KEY_NONE) ck = make_key(sq8_dist_from_e(-key_dist(key), qn, ip, scale_sq), key_id(key));
    keys[j] = ck;
  }
  if (threadIdx.x == 0) {
    s_flag = 0;
    s_thr = 0ull;
  }
  __syncthreads();
  const int r = block_radix_select<MT>(keys, ncand, R, sel, rs);
  unsigned long long mx = 0ull;
  for (int j = threadIdx.x; j < r; j += MT) mx = sel[j] > mx ? sel[j] : mx;
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = t > mx ? t : mx;
  }
  if (lane == 0) atomicMax(&s_thr, mx);
  __syncthreads();
  const uint64_t pad0 = KEY_NONE - (uint64_t)ncand;
  const uint64_t thr = s_thr;
  const float thr_d = thr <= pad0 ? key_dist(thr) : __int_as_float(0x7f800000);
  for (int sg = warp; sg < nseg; sg += MT / 32) {
    bool full = true;
    float emin = __int_as_float(0x7f800000);
    for (int j = lane; j < kseg; j += 32) {
      const uint64_t key = c[(int64_t)sg * ncp + j];
      full = full && key != KEY_NONE;
      if (key != KEY_NONE) emin = fminf(emin, -key_dist(key));
    }
    full = __all_sync(0xffffffffu, full);
    for (int o = 16; o > 0; o >>= 1) emin = fminf(emin, __shfl_xor_sync(0xffffffffu, emin, o));
    // A dropped row has e <= emin, so its distance is at least that of emin.
    if (lane == 0 && full && !(sq8_dist_from_e(emin, qn, ip, scale_sq) > thr_d)) s_flag = 1;
  }
  // ascending, like the integer scan's selection
  for (int j = r + threadIdx.x; j < Rp; j += MT) sel[j] = KEY_NONE;
  __syncthreads();
  if (threadIdx.x == 0) flag[row] = s_flag;
  block_bitonic_sort(sel, Rp);
  for (int j = threadIdx.x; j < R; j += MT)
    out_keys[row * R + j] = sel[j] <= pad0 ? sel[j] : KEY_NONE;
}

}  // namespace

void launch_flat_merge(const uint64_t* cand, int64_t nq, int nseg, int ncp, int kseg, int R,
                       uint64_t* out_keys, int k, const float* qnorm, int metric, float fill_d,
                       float* out_d, int64_t* out_l, int* overflow, cudaStream_t s) {
  if (nq == 0) return;
  MV_REQUIRE(nq <= 0x7fffffffll, MV_ERR_UNSUPPORTED, "too many queries in one batch");
  const int Rp = next_pow2(R);
  const size_t smem = (size_t)(nseg * ncp + Rp) * 8;
  MV_REQUIRE(smem <= 220 * 1024, MV_ERR_UNSUPPORTED, "flat shortlist too large");
  smem_limit(k_flat_merge, smem);
  k_flat_merge<<<(unsigned)nq, MT, smem, s>>>(cand, nseg, ncp, kseg, R, out_keys, k, Rp, qnorm,
                                              metric, fill_d, out_d, out_l, overflow);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv

namespace mv {

void launch_sq8_merge(const uint64_t* cand, int64_t nq, int nseg, int ncp, int kseg, int R,
                      const uint32_t* qnorm, bool ip, float scale_sq, uint64_t* out_keys, int* flag,
                      cudaStream_t s) {
  if (nq == 0) return;
  MV_REQUIRE(nq <= 0x7fffffffll, MV_ERR_UNSUPPORTED, "too many queries in one batch");
  const size_t smem = (size_t)(nseg * ncp + next_pow2(R)) * 8;
  MV_REQUIRE(smem <= 220 * 1024, MV_ERR_UNSUPPORTED, "SQ8 shortlist too large");
  smem_limit(k_sq8_merge, smem);
  k_sq8_merge<<<(unsigned)nq, MT, smem, s>>>(cand, nseg, ncp, kseg, R, qnorm, ip ? 1 : 0, scale_sq,
                                             out_keys, flag);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
