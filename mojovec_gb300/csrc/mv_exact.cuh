// Device arithmetic that reproduces the reference's FP32 operation order.
//
// The reference computes every distance with the SIMD kernels of
// utils/distances.mojo. The plain (drop-in) GPU form must return the same
// FP32 bits, so this header restates their operation order with explicit
// round-to-nearest intrinsics (no contraction, no reassociation):
//
//   l2_distance_simd[W] (distances.mojo:43-143):
//     d < W      -> scalar:  r = r + diff*diff
//     4 accumulators of W lanes over blocks of 4W: acc_a[l] = fma(diff,diff,acc_a[l])
//     s[l] = ((acc0[l] + acc1[l]) + acc2[l]) + acc3[l]
//     W-wide steps: s[l] = fma(diff, diff, s[l])
//     res = reduce_add(s)      (halving tree: lane i += lane i + W/2)
//     W>=32: 16-wide tails, W>=16: 8-wide tails, W>=8: 4-wide tails,
//            each res = res + reduce_add(diff*diff)
//     scalar remainder res = res + diff*diff
//   inner_product_simd[W] (distances.mojo:146-228): same skeleton with
//     fma(x, y, acc) and tails reduce_add(fma(x, y, 0)).
//   l2_distance_short4 / inner_product_short4 (distances.mojo:9-39):
//     d == 4 -> reduce_add of 4 products, else sequential.
#pragma once

#include <cstdint>

#include "mv_kernels.h"

namespace mv {

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// reduce_add over W lanes held in an array.
template <int W>
__device__ __forceinline__ float tree_sum(float* v) {
#pragma unroll
  for (int h = W / 2; h >= 1; h /= 2) {
#pragma unroll
    for (int i = 0; i < h; ++i) v[i] = fadd(v[i], v[i + h]);
  }
  return v[0];
}

// Per-thread l2_distance_simd[W] over two pointers (any address space).
template <int W>
__device__ float l2_simd(const float* x, const float* y, int d) {
  if (d < W) {
    float r = 0.0f;
    for (int i = 0; i < d; ++i) {
      float df = fsub(x[i], y[i]);
      r = fadd(r, fmul(df, df));
    }
    return r;
  }
  float a0[W], a1[W], a2[W], a3[W];
#pragma unroll
  for (int l = 0; l < W; ++l) a0[l] = a1[l] = a2[l] = a3[l] = 0.0f;
  int i = 0;
  for (; i <= d - 4 * W; i += 4 * W) {
#pragma unroll
    for (int l = 0; l < W; ++l) {
      float d0 = fsub(x[i + l], y[i + l]);
      a0[l] = ffma(d0, d0, a0[l]);
      float d1 = fsub(x[i + W + l], y[i + W + l]);
      a1[l] = ffma(d1, d1, a1[l]);
      float d2 = fsub(x[i + 2 * W + l], y[i + 2 * W + l]);
      a2[l] = ffma(d2, d2, a2[l]);
      float d3 = fsub(x[i + 3 * W + l], y[i + 3 * W + l]);
      a3[l] = ffma(d3, d3, a3[l]);
    }
  }
  float s[W];
#pragma unroll
  for (int l = 0; l < W; ++l) s[l] = fadd(fadd(fadd(a0[l], a1[l]), a2[l]), a3[l]);
  for (; i <= d - W; i += W) {
#pragma unroll
    for (int l = 0; l < W; ++l) {
      float df = fsub(x[i + l], y[i + l]);
      s[l] = ffma(df, df, s[l]);
    }
  }
  float res = tree_sum<W>(s);
  if (W >= 32) {
    for (; i <= d - 16; i += 16) {
      float r[16];
#pragma unroll
      for (int l = 0; l < 16; ++l) {
        float df = fsub(x[i + l], y[i + l]);
        r[l] = fmul(df, df);
      }
      res = fadd(res, tree_sum<16>(r));
    }
  }
  if (W >= 16) {
    for (; i <= d - 8; i += 8) {
      float r[8];
#pragma unroll
      for (int l = 0; l < 8; ++l) {
        float df = fsub(x[i + l], y[i + l]);
        r[l] = fmul(df, df);
      }
      res = fadd(res, tree_sum<8>(r));
    }
  }
  if (W >= 8) {
    for (; i <= d - 4; i += 4) {
      float r[4];
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        float df = fsub(x[i + l], y[i + l]);
        r[l] = fmul(df, df);
      }
      res = fadd(res, tree_sum<4>(r));
    }
  }
  for (; i < d; ++i) {
    float df = fsub(x[i], y[i]);
    res = fadd(res, fmul(df, df));
  }
  return res;
}

// Per-thread inner_product_simd[W].
template <int W>
__device__ float ip_simd(const float* x, const float* y, int d) {
  if (d < W) {
    float r = 0.0f;
    for (int i = 0; i < d; ++i) r = fadd(r, fmul(x[i], y[i]));
    return r;
  }
  float p0[W], p1[W], p2[W], p3[W];
#pragma unroll
  for (int l = 0; l < W; ++l) p0[l] = p1[l] = p2[l] = p3[l] = 0.0f;
  int i = 0;
  for (; i <= d - 4 * W; i += 4 * W) {
#pragma unroll
    for (int l = 0; l < W; ++l) {
      p0[l] = ffma(x[i + l], y[i + l], p0[l]);
      p1[l] = ffma(x[i + W + l], y[i + W + l], p1[l]);
      p2[l] = ffma(x[i + 2 * W + l], y[i + 2 * W + l], p2[l]);
      p3[l] = ffma(x[i + 3 * W + l], y[i + 3 * W + l], p3[l]);
    }
  }
  float s[W];
#pragma unroll
  for (int l = 0; l < W; ++l) s[l] = fadd(fadd(fadd(p0[l], p1[l]), p2[l]), p3[l]);
  for (; i <= d - W; i += W) {
#pragma unroll
    for (int l = 0; l < W; ++l) s[l] = ffma(x[i + l], y[i + l], s[l]);
  }
  float res = tree_sum<W>(s);
  if (W >= 32) {
    for (; i <= d - 16; i += 16) {
      float r[16];
#pragma unroll
      for (int l = 0; l < 16; ++l) r[l] = ffma(x[i + l], y[i + l], 0.0f);
      res = fadd(res, tree_sum<16>(r));
    }
  }
  if (W >= 16) {
    for (; i <= d - 8; i += 8) {
      float r[8];
#pragma unroll
      for (int l = 0; l < 8; ++l) r[l] = ffma(x[i + l], y[i + l], 0.0f);
      res = fadd(res, tree_sum<8>(r));
    }
  }
  if (W >= 8) {
    for (; i <= d - 4; i += 4) {
      float r[4];
#pragma unroll
      for (int l = 0; l < 4; ++l) r[l] = ffma(x[i + l], y[i + l], 0.0f);
      res = fadd(res, tree_sum<4>(r));
    }
  }
  for (; i < d; ++i) res = fadd(res, fmul(x[i], y[i]));
  return res;
}

__device__ __forceinline__ float l2_short4(const float* x, const float* y, int d) {
  if (d == 4) {
    float r[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      float df = fsub(x[l], y[l]);
      r[l] = fmul(df, df);
    }
    return tree_sum<4>(r);
  }
  float res = 0.0f;
  for (int i = 0; i < d; ++i) {
    float df = fsub(x[i], y[i]);
    res = fadd(res, fmul(df, df));
  }
  return res;
}

__device__ __forceinline__ float ip_short4(const float* x, const float* y, int d) {
  if (d == 4) {
    float r[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) r[l] = fmul(x[l], y[l]);
    return tree_sum<4>(r);
  }
  float res = 0.0f;
  for (int i = 0; i < d; ++i) res = fadd(res, fmul(x[i], y[i]));
  return res;
}

// PQ sub-distance as ProductQuantizer chooses it (pq.mojo:206-213, 275-292):
// L2: short4 for dsub <= 4 else l2_simd[8]; IP: -(short4 or ip_simd[4]).
__device__ __forceinline__ float pq_sub_l2(const float* x, const float* c, int dsub) {
  return dsub <= 4 ? l2_short4(x, c, dsub) : l2_simd<8>(x, c, dsub);
}
__device__ __forceinline__ float pq_sub_negip(const float* x, const float* c, int dsub) {
  return -(dsub <= 4 ? ip_short4(x, c, dsub) : ip_simd<4>(x, c, dsub));
}

}  // namespace mv
