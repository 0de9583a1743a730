// Per-query ADC tables and table sums of the fast IVF-PQ scan, shared by
// the scan kernels (k_ivfpq_fast.cu, k_ivfpq_scan.cu) so that every kernel
// computes the same FP32 table values and the same sum for a code.
//
// The fast form expands ||q - c - y||^2 as ||q - c||^2 + (||y||^2 + 2<c, y>)
// - 2<q, y> (y the PQ reconstruction of the residual); the table holds
// scale * <q_m, C[m][k]> per subspace m and codeword k (scale -2 for L2,
// -1 for the inner product, index/index_ivf_pq.mojo:316-341).
#pragma once

#include <cuda_fp16.h>

#include <cstdint>

namespace mv {

// Per-query table lut[m][k] = scale * <q_m, C[m][k]>: warp w builds
// subspaces w, w + 8, ...; each lane owns 8 codewords and keeps q_m in
// registers, with the codeword rows read as float4 when dsub is 4 or 8.
// Emits value v of entry (mm, k) through put(index, v).
template <int NT, typename Put>
__device__ __forceinline__ void build_lut(Put put, const float* qv, const float* pq, int M,
                                          int dsub, float scale) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int mm = warp; mm < M; mm += NT / 32) {
    const float* cm = pq + (int64_t)mm * 256 * dsub;
    const float* xm = qv + mm * dsub;
    if (dsub == 8) {
      const float4 qa = *reinterpret_cast<const float4*>(xm);
      const float4 qb = *reinterpret_cast<const float4*>(xm + 4);
      float4 ca[8], cb[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const float* c = cm + (lane + 32 * u) * 8;
        ca[u] = __ldg(reinterpret_cast<const float4*>(c));
        cb[u] = __ldg(reinterpret_cast<const float4*>(c + 4));
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        float dot = qa.x * ca[u].x;
        dot = fmaf(qa.y, ca[u].y, dot);
        dot = fmaf(qa.z, ca[u].z, dot);
        dot = fmaf(qa.w, ca[u].w, dot);
        dot = fmaf(qb.x, cb[u].x, dot);
        dot = fmaf(qb.y, cb[u].y, dot);
        dot = fmaf(qb.z, cb[u].z, dot);
        dot = fmaf(qb.w, cb[u].w, dot);
        put((mm << 8) + lane + 32 * u, scale * dot);
      }
    } else if (dsub == 4) {
      const float4 qa = *reinterpret_cast<const float4*>(xm);
      float4 ca[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) ca[u] = __ldg(reinterpret_cast<const float4*>(cm + (lane + 32 * u) * 4));
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        float dot = qa.x * ca[u].x;
        dot = fmaf(qa.y, ca[u].y, dot);
        dot = fmaf(qa.z, ca[u].z, dot);
        dot = fmaf(qa.w, ca[u].w, dot);
        put((mm << 8) + lane + 32 * u, scale * dot);
      }
    } else {
      for (int u = 0; u < 8; ++u) {
        const float* c = cm + (lane + 32 * u) * dsub;
        float dot = 0.0f;
        for (int t = 0; t < dsub; ++t) dot = fmaf(xm[t], c[t], dot);
        put((mm << 8) + lane + 32 * u, scale * dot);
      }
    }
  }
}

// The same table from an FP16 copy of the codebook scaled by a power of two
// (pq16 = s * pq, inv = 1 / s; dsub 4 or 8): half the bytes read per query.
template <int NT, typename Put>
__device__ __forceinline__ void build_lut16(Put put, const float* qv, const __half* pq16, int M,
                                            int dsub, float scale) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int mm = warp; mm < M; mm += NT / 32) {
    const __half* cm = pq16 + (int64_t)mm * 256 * dsub;
    const float* xm = qv + mm * dsub;
    if (dsub == 8) {
      const float4 qa = *reinterpret_cast<const float4*>(xm);
      const float4 qb = *reinterpret_cast<const float4*>(xm + 4);
      uint4 cw[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) cw[u] = __ldg(reinterpret_cast<const uint4*>(cm + (lane + 32 * u) * 8));
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const float2 c0 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].x));
        const float2 c1 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].y));
        const float2 c2 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].z));
        const float2 c3 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].w));
        float dot = qa.x * c0.x;
        dot = fmaf(qa.y, c0.y, dot);
        dot = fmaf(qa.z, c1.x, dot);
        dot = fmaf(qa.w, c1.y, dot);
        dot = fmaf(qb.x, c2.x, dot);
        dot = fmaf(qb.y, c2.y, dot);
        dot = fmaf(qb.z, c3.x, dot);
        dot = fmaf(qb.w, c3.y, dot);
        put((mm << 8) + lane + 32 * u, scale * dot);
      }
    } else {  // dsub == 4
      const float4 qa = *reinterpret_cast<const float4*>(xm);
      uint2 cw[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) cw[u] = __ldg(reinterpret_cast<const uint2*>(cm + (lane + 32 * u) * 4));
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const float2 c0 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].x));
        const float2 c1 = __half22float2(*reinterpret_cast<const __half2*>(&cw[u].y));
        float dot = qa.x * c0.x;
        dot = fmaf(qa.y, c0.y, dot);
        dot = fmaf(qa.z, c1.x, dot);
        dot = fmaf(qa.w, c1.y, dot);
        put((mm << 8) + lane + 32 * u, scale * dot);
      }
    }
  }
}

// Sum of the M table entries of one code; four partial sums break the
// dependency chain (the fast form does not reproduce the reference's order).
template <typename T>
__device__ __forceinline__ float lut_val(const T* lut, int i) {
  if constexpr (sizeof(T) == 2) return __half2float(lut[i]);
  else return lut[i];
}

template <typename T>
__device__ __forceinline__ float adc_fast(const T* lut, const uint8_t* code, int M, float acc) {
  float p[4] = {acc, 0.0f, 0.0f, 0.0f};
  if ((M & 15) == 0) {
    for (int m0 = 0; m0 < M; m0 += 16) {
      const uint4 v = *reinterpret_cast<const uint4*>(code + m0);
      const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int b = 0; b < 4; ++b) p[b] += lut_val(lut, ((m0 + 4 * i + b) << 8) + ((w[i] >> (8 * b)) & 255u));
    }
  } else if ((M & 7) == 0) {
    for (int m0 = 0; m0 < M; m0 += 8) {
      const uint2 v = *reinterpret_cast<const uint2*>(code + m0);
      const uint32_t w[2] = {v.x, v.y};
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int b = 0; b < 4; ++b) p[b] += lut_val(lut, ((m0 + 4 * i + b) << 8) + ((w[i] >> (8 * b)) & 255u));
    }
  } else {
    for (int m = 0; m < M; ++m) p[m & 3] += lut_val(lut, (m << 8) + code[m]);
  }
  return (p[0] + p[1]) + (p[2] + p[3]);
}

}  // namespace mv
