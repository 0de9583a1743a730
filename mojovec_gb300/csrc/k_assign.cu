// Certified exact selections on the tensor cores.
//
// The plain form must return the reference's own FP32 results: the nearest
// centroid of a row (index/index_flat.mojo:292-310 with k = 1 for the coarse
// quantizer; clustering/kmeans.mojo:123-141 in k-means) and the Flat top-k
// (index/index_flat.mojo:260-325), with the smaller index on equal
// distances. Here the BF16 tensor-core top-k GEMM (k_umma_topk) proposes
// candidates, their distances are recomputed with the reference's FP32
// operation order (l2_simd<8> / -ip_simd<8>), and the bound of mv_cert.cuh
// decides whether any row outside the candidates could still rank ahead.
// Selections the bound does not settle (and those with NaN or huge
// distances) are listed for the exact SIMT scan, so the result always equals
// the exact one.
#include <cuda_bf16.h>

#include "mv_cert.cuh"
#include "mv_exact.cuh"
#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"

namespace mv {
namespace {

// cert[0] = B^2 bound: max of the FP32 norms of the BF16 rows with the
// summation slack (rounded up), or -1 when a norm is NaN or infinite.
__global__ void k_max_norm(const float* __restrict__ norms, int64_t n, int d,
                           float* __restrict__ out) {
  __shared__ float part[32];
  float m = 0.0f;
  bool bad = false;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const float v = norms[i];
    if (!(v <= 3.0e38f)) bad = true;  // NaN or inf
    else m = fmaxf(m, v);
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  bad = __any_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = bad ? -1.0f : m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float r = 0.0f;
    bool anybad = false;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      if (part[w] < 0.0f) anybad = true;
      r = fmaxf(r, part[w]);
    }
    *out = anybad ? -1.0f : __fmul_ru(r, __fadd_ru(1.0f, __fmul_ru((float)(d + 1), 0x1p-23f)));
  }
}

// out = max over rows of an upper bound on ||y - bf16(y)|| (bits of a
// non-negative float, zeroed by the caller), one warp per row: the
// differences are exact in FP32, their squares and sums rounded up.
__global__ void k_resid_max(const float* __restrict__ rows, int64_t n, int d,
                            unsigned* __restrict__ out) {
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  float s = 0.0f;
  for (int j = lane; j < d; j += 32) {
    const float v = rows[row * d + j];
    const float r = __fsub_rn(v, __bfloat162float(__float2bfloat16_rn(v)));
    s = __fadd_ru(s, __fmul_ru(r, r));
  }
  for (int o = 16; o > 0; o >>= 1) s = __fadd_ru(s, __shfl_xor_sync(0xffffffffu, s, o));
  if (lane == 0) {
    const float v = s != s ? 1e30f : __fsqrt_ru(s);  // NaN: no certificate
    atomicMax(out, __float_as_uint(v));
  }
}

__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}

// Nearest centroid, one warp per row.
template <bool IP>
__global__ void k_assign_certify(const float* __restrict__ x, int64_t n, int d,
                                 const float* __restrict__ cent, int nlist,
                                 const uint64_t* __restrict__ cand, int ncand, int kc,
                                 const float* __restrict__ cert, int32_t* __restrict__ assign,
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
    // K: the kc-th smallest candidate key (the largest a full heap keeps)
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
    const CertNorms cn = cert_norms(xr, d);
    const float B2 = cert[0], rmax = cert[1];
    if (valid < kc || prev == KEY_NONE || !cert_inputs_ok(cn, B2, rmax)) {
      ok = false;
    } else {
      const float K = key_dist(prev);
      const float lower = IP ? cert_lower_ip(cn, B2, rmax, K, d) : cert_lower_l2(cn, B2, rmax, K, d);
      ok = lower > best;
    }
  }
  if (lane == 0) {
    assign[row] = bi == 0x7fffffff ? 0 : bi;
    if (mind) mind[row] = best;
    if (!ok) flagged[atomicAdd(nflag, 1)] = row;
  }
}

// In-place ascending bitonic sort of n keys (a power of two) by one warp.
__device__ __forceinline__ void warp_sort_keys(uint64_t* a, int n) {
  const int lane = threadIdx.x & 31;
  for (int k = 2; k <= n; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < n; i += 32) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const uint64_t x = a[i], y = a[ixj];
          if ((x > y) == ((i & k) == 0)) {
            a[i] = y;
            a[ixj] = x;
          }
        }
      }
      __syncwarp();
    }
}

// The P nearest centroids of each query (the coarse quantizer search with
// k = nprobe, index/index_flat.mojo:292-310), one warp per query: the
// candidates' reference distances, the P smallest (distance, list) keys in
// ascending order, and the bound for the centroids outside the candidates
// against the P-th. Open queries are appended to flagged[].
constexpr int TP_WARPS = 4, TP_CAP = 256;

template <bool IP>
__global__ void __launch_bounds__(TP_WARPS * 32)
    k_topp_certify(const float* __restrict__ x, int64_t n, int d, const float* __restrict__ cent,
                   int nlist, const uint64_t* __restrict__ cand, int ncand, int kc, int P,
                   const float* __restrict__ cert, int32_t* __restrict__ probes,
                   int64_t* __restrict__ flagged, int* __restrict__ nflag) {
  __shared__ uint64_t bufs[TP_WARPS][TP_CAP];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * TP_WARPS + warp;
  if (row >= n) return;  // warps are independent
  uint64_t* B = bufs[warp];
  const float* xr = x + row * d;
  const uint64_t* ck = cand + row * ncand;
  int np2 = 32;
  while (np2 < ncand) np2 <<= 1;
  bool bad = false;
  int valid = 0;
  for (int c = lane; c < np2; c += 32) {
    uint64_t e = KEY_NONE - (uint64_t)c;  // distinct padding keys sort last
    if (c < ncand) {
      const uint64_t key = ck[c];
      if (key != KEY_NONE && key_id(key) < (uint32_t)nlist) {
        const uint32_t ci = key_id(key);
        const float* yr = cent + (int64_t)ci * d;
        const float r = IP ? -ip_simd<8>(xr, yr, d) : l2_simd<8>(xr, yr, d);
        if (!(r < 1e38f && r > -1e38f)) bad = true;  // NaN, inf or huge
        e = make_key(r, ci);
        ++valid;
      }
    }
    B[c] = e;
  }
  for (int o = 16; o > 0; o >>= 1) valid += __shfl_xor_sync(0xffffffffu, valid, o);
  bad = __any_sync(0xffffffffu, bad);
  __syncwarp();
  warp_sort_keys(B, np2);
  bool ok = !bad && valid >= P;
  if (ok && valid < nlist) {
    uint64_t prev = 0;  // K: the kc-th smallest candidate key
    for (int t = 0; t < kc; ++t) {
      uint64_t m = KEY_NONE;
      for (int c = lane; c < ncand; c += 32) {
        const uint64_t key = ck[c];
        if (key == KEY_NONE || key_id(key) >= (uint32_t)nlist) continue;
        if ((t == 0 || key > prev) && key < m) m = key;
      }
      prev = warp_min_u64(m);
    }
    const CertNorms cn = cert_norms(xr, d);
    const float B2 = cert[0], rmax = cert[1];
    if (valid < kc || prev == KEY_NONE || !cert_inputs_ok(cn, B2, rmax)) {
      ok = false;
    } else {
      const float K = key_dist(prev);
      const float lower = IP ? cert_lower_ip(cn, B2, rmax, K, d) : cert_lower_l2(cn, B2, rmax, K, d);
      ok = lower > key_dist(B[P - 1]);
    }
  }
  for (int p = lane; p < P; p += 32) probes[row * P + p] = (int32_t)key_id(B[p]);
  if (!ok && lane == 0) flagged[atomicAdd(nflag, 1)] = row;
}

// Flat top-k, one CTA per query over its shortlist of R approximate keys
// (the R smallest of the GEMM's candidates, KEY_NONE padded): the rows are
// staged in shared memory (stride d + 1, so thread t reading row t touches
// its own bank) in chunks of `chunk` rows, each thread computes one row's
// reference distance, the k smallest (distance, row) keys are selected and
// written, and the certificate compares the k-th with the bound for the
// rows outside the shortlist. flag[q] = 1 when it does not settle the query
// (the host recomputes those with the exact scan).
constexpr int FC_THREADS = 128, FC_CHUNK_MAX = 64;

template <bool IP>
__global__ void __launch_bounds__(FC_THREADS)
    k_flat_certify(const float* __restrict__ q, int d, const float* __restrict__ rows, int64_t nb,
                   const uint64_t* __restrict__ skeys, int R, int k, int chunk,
                   const float* __restrict__ cert, const int* __restrict__ over,
                   float* __restrict__ out_d, int64_t* __restrict__ out_l,
                   int* __restrict__ flag) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int stride = d + 1;
  float* qv = reinterpret_cast<float*>(smraw);
  float* tile = qv + d;  // chunk x (d + 1)
  uint64_t* ek = reinterpret_cast<uint64_t*>(
      smraw + (((size_t)d + (size_t)chunk * stride) * 4 + 15) / 16 * 16);  // R
  uint64_t* outb = ek + R;                                                  // next_pow2(k)
  __shared__ RadixScratch rs;
  __shared__ unsigned long long s_kmax;
  __shared__ int s_valid, s_bad;
  __shared__ CertNorms s_cn;
  const int64_t row = blockIdx.x;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint64_t* sk = skeys + row * R;
  for (int j = tid; j < d; j += FC_THREADS) qv[j] = q[row * d + j];
  if (tid == 0) {
    s_kmax = 0ull;
    s_valid = 0;
    s_bad = 0;
  }
  __syncthreads();
  if (warp == 0) {
    const CertNorms cn = cert_norms(qv, d);
    if (lane == 0) s_cn = cn;
  }
  for (int c0 = 0; c0 < R; c0 += chunk) {
    const int n = min(chunk, R - c0);
    // stage the chunk's rows, one warp per row, coalesced
    for (int i = warp; i < n; i += FC_THREADS / 32) {
      const uint64_t key = sk[c0 + i];
      const int64_t pos = key == KEY_NONE ? -1 : (int64_t)key_id(key);
      if (pos >= 0 && pos < nb)
        for (int j = lane; j < d; j += 32) tile[i * stride + j] = rows[pos * d + j];
    }
    __syncthreads();
    for (int i = tid; i < n; i += FC_THREADS) {
      const uint64_t key = sk[c0 + i];
      const int64_t pos = key == KEY_NONE ? -1 : (int64_t)key_id(key);
      uint64_t e = KEY_NONE - (uint64_t)(c0 + i);  // distinct padding keys
      if (pos >= 0 && pos < nb) {
        const float* yr = tile + i * stride;
        const float r = IP ? -ip_simd<8>(qv, yr, d) : l2_simd<8>(qv, yr, d);
        if (!(r < 1e38f && r > -1e38f)) atomicExch(&s_bad, 1);  // NaN, inf or huge
        e = make_key(r, (uint32_t)pos);
        atomicMax(&s_kmax, (unsigned long long)key);
        atomicAdd(&s_valid, 1);
      }
      ek[c0 + i] = e;
    }
    __syncthreads();  // the tile is reused by the next chunk
  }
  const int kp = next_pow2(k);
  const int r = block_radix_select<FC_THREADS>(ek, R, k, outb, rs);
  for (int j = r + tid; j < kp; j += FC_THREADS) outb[j] = KEY_NONE;
  __syncthreads();
  block_bitonic_sort(outb, kp);
  const int valid = s_valid;
  for (int i = tid; i < k; i += FC_THREADS) {
    const uint64_t key = outb[i];
    float dd = 0.0f;  // index_flat.mojo:232-238: unfilled slots 0.0 / -1
    int64_t ll = -1;
    if (i < valid && key < KEY_NONE - (uint64_t)R) {
      dd = key_dist(key);
      if (IP) dd = -dd;
      ll = (int64_t)key_id(key);
    }
    out_d[row * k + i] = dd;
    out_l[row * k + i] = ll;
  }
  if (tid == 0) {
    bool ok = !s_bad && !(over && over[row]);
    if (ok && valid >= R) {  // rows outside the shortlist exist: bound them
      const float B2 = cert[0], rmax = cert[1];
      const CertNorms cn = s_cn;
      if (!cert_inputs_ok(cn, B2, rmax) || valid < k) {
        ok = false;
      } else {
        const float K = key_dist((uint64_t)s_kmax);
        const float lower = IP ? cert_lower_ip(cn, B2, rmax, K, d) : cert_lower_l2(cn, B2, rmax, K, d);
        ok = lower > key_dist(outb[k - 1]);
      }
    }
    flag[row] = ok ? 0 : 1;
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

void launch_cert_bounds(const float* norms, const float* rows, int64_t n, int d, float* cert,
                        cudaStream_t s) {
  k_max_norm<<<1, 1024, 0, s>>>(norms, n, d, cert);
  MV_CHECK_CUDA(cudaMemsetAsync(cert + 1, 0, sizeof(float), s));
  if (n > 0)
    k_resid_max<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(rows, n, d,
                                                         reinterpret_cast<unsigned*>(cert + 1));
  count_launch();
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_assign_certify(const float* x, int64_t n, int d, const float* cent, int nlist, int metric,
                           const uint64_t* cand, int ncand, int kc, const float* cert,
                           int32_t* assign, float* mind, int64_t* flagged, int* nflag,
                           cudaStream_t s) {
  if (n == 0) return;
  const unsigned grid = (unsigned)((n + 7) / 8);
  if (metric == MV_METRIC_IP)
    k_assign_certify<true><<<grid, 256, 0, s>>>(x, n, d, cent, nlist, cand, ncand, kc, cert,
                                                assign, mind, flagged, nflag);
  else
    k_assign_certify<false><<<grid, 256, 0, s>>>(x, n, d, cent, nlist, cand, ncand, kc, cert,
                                                 assign, mind, flagged, nflag);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_topp_certify(const float* x, int64_t n, int d, const float* cent, int nlist, int metric,
                         const uint64_t* cand, int ncand, int kc, int P, const float* cert,
                         int32_t* probes, int64_t* flagged, int* nflag, cudaStream_t s) {
  if (n == 0) return;
  MV_REQUIRE(ncand <= TP_CAP && P >= 1 && P <= kc, MV_ERR_INTERNAL, "top-P certify: bad sizes");
  const unsigned grid = (unsigned)((n + TP_WARPS - 1) / TP_WARPS);
  if (metric == MV_METRIC_IP)
    k_topp_certify<true><<<grid, TP_WARPS * 32, 0, s>>>(x, n, d, cent, nlist, cand, ncand, kc, P,
                                                        cert, probes, flagged, nflag);
  else
    k_topp_certify<false><<<grid, TP_WARPS * 32, 0, s>>>(x, n, d, cent, nlist, cand, ncand, kc, P,
                                                         cert, probes, flagged, nflag);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

// Rows staged per chunk: up to 64, fewer for long rows.
int flat_certify_chunk(int d, int R, int k) {
  const long room = 160l * 1024 - (long)d * 4 - (long)(R + next_pow2(k)) * 8 - 16;
  return (int)std::max(1l, std::min((long)FC_CHUNK_MAX, room / ((long)(d + 1) * 4)));
}

size_t flat_certify_smem(int d, int R, int k) {
  return ((size_t)d + (size_t)flat_certify_chunk(d, R, k) * (d + 1)) * 4 + 16 +
         (size_t)(R + next_pow2(k)) * 8;
}

void launch_flat_certify(const float* q, int64_t nq, int d, int metric, const float* rows,
                         int64_t nb, const uint64_t* skeys, int R, int k, const float* cert,
                         const int* over, float* out_d, int64_t* out_l, int* flag,
                         cudaStream_t s) {
  if (nq == 0) return;
  const size_t smem = flat_certify_smem(d, R, k);
  MV_REQUIRE(smem <= 200 * 1024, MV_ERR_UNSUPPORTED, "flat certify: d or shortlist too large");
  const int chunk = flat_certify_chunk(d, R, k);
  if (metric == MV_METRIC_IP) {
    smem_limit(k_flat_certify<true>, smem);
    k_flat_certify<true><<<(unsigned)nq, FC_THREADS, smem, s>>>(q, d, rows, nb, skeys, R, k, chunk,
                                                               cert, over, out_d, out_l, flag);
  } else {
    smem_limit(k_flat_certify<false>, smem);
    k_flat_certify<false><<<(unsigned)nq, FC_THREADS, smem, s>>>(q, d, rows, nb, skeys, R, k,
                                                                chunk, cert, over, out_d, out_l,
                                                                flag);
  }
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
