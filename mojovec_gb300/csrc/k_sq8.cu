// SQ8 codec, SQ8 distance tiles, the exact FP32 rerank and FP64 row
// normalisation.
//
// SQ8 follows quantization/sq8.mojo and index/index_flat_sq8.mojo:
//   encode (sq8.mojo:13-38): L2 u8 = clamp(round((x - min) * inv), 0, 255),
//     IP s8 = clamp(round(x * inv), -127, 127), norm = sum code^2 (u32);
//   distance (sq8.mojo:62-79): L2 Float32(u32(max(|q|^2 + |x|^2 - 2 q.x, 0)))
//     * scale^2, IP -Float32(q.x) * scale^2.
// The dots are integer (dp4a on 32-bit words of 4 codes), so any summation
// order gives the reference's value. Rows are stored dpad (multiple of 16)
// bytes wide with zero padding, which leaves dots and norms unchanged.
#include "mv_exact.cuh"
#include <cuda_bf16.h>

#include "mv_internal.h"
#include "mv_kernels.h"
#include "mv_select.cuh"

namespace mv {
namespace {

__device__ __forceinline__ uint32_t f_ord(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void k_minmax(const float* __restrict__ x, int64_t n, unsigned int* __restrict__ out2) {
  uint32_t lo = 0xffffffffu, hi = 0u;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t o = f_ord(x[i]);
    lo = min(lo, o);
    hi = max(hi, o);
  }
  for (int s = 16; s > 0; s >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, s));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, s));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&out2[0], lo);
    atomicMax(&out2[1], hi);
  }
}

__global__ void k_minmax_init(unsigned int* v) {
  v[0] = 0xffffffffu;
  v[1] = 0u;
}

__global__ void k_ord_to_float(unsigned int* v) {
  for (int i = 0; i < 2; ++i) {
    uint32_t o = v[i];
    uint32_t u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
    v[i] = u;
  }
}

// One warp per row.
__global__ void k_sq8_encode(const float* __restrict__ x, int64_t n, int d, int dpad,
                             float minimum, float inv, int symmetric, uint8_t* __restrict__ codes,
                             uint32_t* __restrict__ norms) {
  const int lane = threadIdx.x & 31;
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= n) return;
  const float* xr = x + row * d;
  uint8_t* cr = codes + row * dpad;
  uint32_t norm = 0;
  for (int j = lane; j < dpad; j += 32) {
    uint8_t code = 0;
    if (j < d) {
      if (symmetric) {
        float scaled = roundf(fmul(xr[j], inv));
        float cl = fminf(fmaxf(scaled, -127.0f), 127.0f);
        int8_t c = (int8_t)(int)cl;
        code = (uint8_t)c;
        int32_t w = c;
        norm += (uint32_t)(w * w);
      } else {
        float scaled = roundf(fmul(fsub(xr[j], minimum), inv));
        float cl = fminf(fmaxf(scaled, 0.0f), 255.0f);
        code = (uint8_t)(int)cl;
        norm += (uint32_t)code * (uint32_t)code;
      }
    }
    cr[j] = code;
  }
  for (int s = 16; s > 0; s >>= 1) norm += __shfl_xor_sync(0xffffffffu, norm, s);
  if (lane == 0) norms[row] = norm;
}

constexpr int TB = 64;
constexpr int NT = 256;

__device__ __forceinline__ int wswz(int w, int r) { return w * TB + (r ^ (((w >> 2) & 7) << 2)); }

__device__ __forceinline__ void stage_codes(uint32_t* S, const uint8_t* C, int64_t nrows, int dpad,
                                            int64_t row0) {
  const int words = dpad >> 2;
  const int total = TB * words;
  for (int e = threadIdx.x; e < total; e += NT) {
    int r = e / words;
    int w = e - r * words;
    int64_t gr = row0 + r;
    S[wswz(w, r)] = (gr < nrows) ? reinterpret_cast<const uint32_t*>(C + gr * dpad)[w] : 0u;
  }
}

template <bool IP>
__global__ void __launch_bounds__(NT)
    k_sq8_matrix(const uint8_t* __restrict__ qc, const uint32_t* __restrict__ qn, int64_t nq,
                 const uint8_t* __restrict__ bc, const uint32_t* __restrict__ bn, int64_t nb,
                 int dpad, float scale_sq, float* __restrict__ D, int64_t ldd) {
  extern __shared__ uint32_t smw[];
  const int words = dpad >> 2;
  uint32_t* Qs = smw;
  uint32_t* Bs = smw + TB * words;
  const int64_t row0 = (int64_t)blockIdx.y * TB;
  const int64_t col0 = (int64_t)blockIdx.x * TB;
  stage_codes(Qs, qc, nq, dpad, row0);
  stage_codes(Bs, bc, nb, dpad, col0);
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int rx = ty * 4, cy = tx * 4;
  int acc[16];
#pragma unroll
  for (int p = 0; p < 16; ++p) acc[p] = 0;
  for (int w = 0; w < words; ++w) {
    uint4 a = *reinterpret_cast<const uint4*>(&Qs[wswz(w, rx)]);
    uint4 b = *reinterpret_cast<const uint4*>(&Bs[wswz(w, cy)]);
    uint32_t av[4] = {a.x, a.y, a.z, a.w};
    uint32_t bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (IP)
          acc[i * 4 + j] = __dp4a((int)av[i], (int)bv[j], acc[i * 4 + j]);
        else
          acc[i * 4 + j] = (int)__dp4a(av[i], bv[j], (unsigned)acc[i * 4 + j]);
      }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int64_t r = row0 + rx + i;
    if (r >= nq) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int64_t c = col0 + cy + j;
      if (c >= nb) continue;
      float dist;
      if (IP) {
        dist = fmul(-__int2float_rn(acc[i * 4 + j]), scale_sq);
      } else {
        int64_t dd = (int64_t)qn[r] + (int64_t)bn[c] - 2 * (int64_t)(uint32_t)acc[i * 4 + j];
        uint32_t u = (uint32_t)(dd > 0 ? dd : 0);
        dist = fmul(__uint2float_rn(u), scale_sq);
      }
      D[r * ldd + c] = dist;
    }
  }
}

// Warp-cooperative l2_distance_simd[64] / inner_product_simd[64]
// (utils/distances.mojo:43-228 at W = 64): lane t owns SIMD lanes t and
// t + 32; the 64-lane reduce_add first folds lane t + 32 into t, then
// halves through shuffles.
template <bool IP>
__device__ float warp_simd64(const float* x, const float* y, int d) {
  const int lane = threadIdx.x & 31;
  const unsigned FULL = 0xffffffffu;
  auto prod = [&](int e) -> float {
    if (IP) return ffma(x[e], y[e], 0.0f);
    float df = fsub(x[e], y[e]);
    return fmul(df, df);
  };
  if (d < 64) {
    float r = 0.0f;
    if (lane == 0) {
      for (int i = 0; i < d; ++i) {
        float t;
        if (IP) {
          t = fmul(x[i], y[i]);
        } else {
          float df = fsub(x[i], y[i]);
          t = fmul(df, df);
        }
        r = fadd(r, t);
      }
    }
    return __shfl_sync(FULL, r, 0);
  }
  float a[4][2];
#pragma unroll
  for (int u = 0; u < 4; ++u) a[u][0] = a[u][1] = 0.0f;
  int i = 0;
  for (; i <= d - 256; i += 256) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        int e = i + 64 * u + lane + 32 * h;
        if (IP) {
          a[u][h] = ffma(x[e], y[e], a[u][h]);
        } else {
          float df = fsub(x[e], y[e]);
          a[u][h] = ffma(df, df, a[u][h]);
        }
      }
  }
  float s[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) s[h] = fadd(fadd(fadd(a[0][h], a[1][h]), a[2][h]), a[3][h]);
  for (; i <= d - 64; i += 64) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int e = i + lane + 32 * h;
      if (IP) {
        s[h] = ffma(x[e], y[e], s[h]);
      } else {
        float df = fsub(x[e], y[e]);
        s[h] = ffma(df, df, s[h]);
      }
    }
  }
  float v = fadd(s[0], s[1]);
  for (int h = 16; h >= 1; h >>= 1) {
    float o = __shfl_down_sync(FULL, v, h);
    if (lane < h) v = fadd(v, o);
  }
  float res = __shfl_sync(FULL, v, 0);
  // 16-, 8- and 4-wide tails: each adds reduce_add(products) to res.
  for (int width = 16; width >= 4; width >>= 1) {
    for (; i <= d - width; i += width) {
      float r = (lane < width) ? prod(i + lane) : 0.0f;
      for (int h = width >> 1; h >= 1; h >>= 1) {
        float o = __shfl_down_sync(FULL, r, h);
        if (lane < h) r = fadd(r, o);
      }
      res = fadd(res, __shfl_sync(FULL, r, 0));
    }
  }
  float tail = res;
  if (lane == 0) {
    for (; i < d; ++i) {
      float t;
      if (IP) {
        t = fmul(x[i], y[i]);
      } else {
        float df = fsub(x[i], y[i]);
        t = fmul(df, df);
      }
      tail = fadd(tail, t);
    }
  }
  return __shfl_sync(FULL, tail, 0);
}

constexpr int RR_THREADS = 256;

__global__ void __launch_bounds__(RR_THREADS)
    k_rerank_simd64(const float* __restrict__ q, int d, const float* __restrict__ base, int64_t nb,
                    int metric, const int64_t* __restrict__ cand, int ncand, int k, int bufcap,
                    uint64_t* __restrict__ out_keys) {
  extern __shared__ uint64_t skeys[];
  __shared__ int cnt;
  __shared__ uint64_t thr;
  const int64_t row = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = RR_THREADS / 32;
  BlockTopK sel;
  sel.init(skeys, &cnt, &thr, k, bufcap);
  const float* qp = q + row * d;
  for (int c0 = 0; c0 < ncand; c0 += nw) {
    int c = c0 + warp;
    if (c < ncand) {
      int64_t id = cand[row * ncand + c];
      if (id >= 0 && id < nb) {  // -1 marks an empty slot
        const float* bp = base + id * d;
        float dist = metric == MV_METRIC_L2 ? warp_simd64<false>(qp, bp, d)
                                           : -warp_simd64<true>(qp, bp, d);
        if (lane == 0) sel.push(make_key(dist, (uint32_t)id));
      }
    }
    sel.end_round();
  }
  sel.finish();
  for (int i = threadIdx.x; i < k; i += RR_THREADS) out_keys[row * k + i] = skeys[i];
}

// _normalize_vectors (api/collection_vector_query.mojo:24-46): one thread
// per row, FP64 sequential sum of squares, inverse = 1 / sqrt in FP64.
__global__ void k_normalize(const float* __restrict__ x, int64_t n, int d, float* __restrict__ out,
                            int32_t* __restrict__ bad) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const float* xr = x + r * d;
  double sq = 0.0;
  for (int j = 0; j < d; ++j) {
    float v = xr[j];
    if (!isfinite(v)) {
      atomicMax(bad, 1);
      return;
    }
    double w = (double)v;
    sq = __dadd_rn(sq, __dmul_rn(w, w));
  }
  if (!(sq > 0.0)) {
    atomicMax(bad, 2);
    return;
  }
  double inv = __ddiv_rn(1.0, __dsqrt_rn(sq));
  for (int j = 0; j < d; ++j) out[r * d + j] = __double2float_rn(__dmul_rn((double)xr[j], inv));
}

}  // namespace

void launch_minmax(const float* x, int64_t n, float* out2, cudaStream_t s) {
  k_minmax_init<<<1, 1, 0, s>>>(reinterpret_cast<unsigned int*>(out2));
  count_launch();
  if (n > 0) {
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
    k_minmax<<<blocks, 256, 0, s>>>(x, n, reinterpret_cast<unsigned int*>(out2));
    count_launch();
  }
  k_ord_to_float<<<1, 1, 0, s>>>(reinterpret_cast<unsigned int*>(out2));
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

// SQ8 codes -> zero-padded BF16 rows (kp wide) for the tensor-core scan:
// u8 codes (L2) as 0..255, s8 codes (IP) as -127..127, both exact in BF16;
// norms (integer sums of squares) as FP32, exact below 2^24.
__global__ void k_sq8_codes_to_bf16(const uint8_t* __restrict__ codes, int64_t n, int d, int dpad,
                                    int kp, int symmetric, const uint32_t* __restrict__ norms,
                                    __nv_bfloat16* __restrict__ out, float* __restrict__ fnorms) {
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  for (int j = lane; j < kp; j += 32) {
    float v = 0.0f;
    if (j < d) {
      const uint8_t c = codes[row * dpad + j];
      v = symmetric ? (float)(int8_t)c : (float)c;
    }
    out[row * kp + j] = __float2bfloat16_rn(v);
  }
  if (lane == 0 && fnorms) fnorms[row] = (float)norms[row];
}

void launch_sq8_codes_to_bf16(const uint8_t* codes, int64_t n, int d, int dpad, int kp,
                              bool symmetric, const uint32_t* norms, __nv_bfloat16* out,
                              float* fnorms, cudaStream_t s) {
  if (n == 0) return;
  k_sq8_codes_to_bf16<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(codes, n, d, dpad, kp,
                                                              symmetric ? 1 : 0, norms, out, fnorms);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_sq8_encode(const float* x, int64_t n, int d, int dpad, float minimum, float inv_scale,
                       bool symmetric, uint8_t* codes, uint32_t* norms, cudaStream_t s) {
  if (n == 0) return;
  k_sq8_encode<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(x, n, d, dpad, minimum, inv_scale,
                                                       symmetric ? 1 : 0, codes, norms);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_sq8_matrix(const uint8_t* qc, const uint32_t* qn, int64_t nq, const uint8_t* bc,
                       const uint32_t* bn, int64_t nb, int dpad, bool ip, float scale_sq,
                       float* D, int64_t ldd, cudaStream_t s) {
  if (nq == 0 || nb == 0) return;
  size_t smem = (size_t)2 * TB * dpad;
  MV_REQUIRE(smem <= 200 * 1024, MV_ERR_UNSUPPORTED, "SQ8 tile: dimension too large");
  MV_REQUIRE((nq + TB - 1) / TB <= 65535, MV_ERR_UNSUPPORTED, "too many queries in one call");
  dim3 grid((unsigned)((nb + TB - 1) / TB), (unsigned)((nq + TB - 1) / TB));
  if (ip) {
    smem_limit(k_sq8_matrix<true>, smem);
    k_sq8_matrix<true><<<grid, NT, smem, s>>>(qc, qn, nq, bc, bn, nb, dpad, scale_sq, D, ldd);
  } else {
    smem_limit(k_sq8_matrix<false>, smem);
    k_sq8_matrix<false><<<grid, NT, smem, s>>>(qc, qn, nq, bc, bn, nb, dpad, scale_sq, D, ldd);
  }
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_rerank_simd64(const float* q, int64_t nq, int d, const float* base, int64_t nb, int metric,
                          const int64_t* cand, int ncand, int k, uint64_t* out_keys,
                          cudaStream_t s) {
  if (nq == 0) return;
  const int bufcap = 512;
  size_t smem = (size_t)BlockTopK::smem_keys(k, bufcap) * 8;
  MV_REQUIRE(smem <= 200 * 1024, MV_ERR_UNSUPPORTED, "rerank: k too large");
  smem_limit(k_rerank_simd64, smem);
  k_rerank_simd64<<<(unsigned)nq, RR_THREADS, smem, s>>>(q, d, base, nb, metric, cand, ncand, k,
                                                          bufcap, out_keys);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_normalize(const float* x, int64_t n, int d, float* out, int32_t* bad, cudaStream_t s) {
  if (n == 0) return;
  k_normalize<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(x, n, d, out, bad);
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
