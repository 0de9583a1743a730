// Lower bounds on the reference FP32 distance of a row that the BF16
// tensor-core top-k GEMM (k_umma_topk) did not keep as a candidate.
//
// Notation: q a query, y a base row or centroid, bq and by the two rounded
// to BF16 (round to nearest); X = ||bq||, rq = ||q - bq||, B an upper bound
// on ||by|| over all rows, rmax an upper bound on ||y - by||. The GEMM ranks
// row y by its key kd = fl(||by||^2 - 2 acc) (L2; ||by||^2 summed in FP32)
// or kd = -acc (IP), acc the tensor core's FP32 sum of the exact products
// bq_i * by_i. Every row it did not keep has kd >= K, the largest key it
// kept (the caller passes that K). Error terms:
//   * ||by||^2 in FP32 and the final rounding of kd: (d + 1) 2^-23 B^2;
//   * acc: each of the d FP32 additions may lose 2^-22 of the running sum
//     of |products| (twice the round-to-nearest bound, allowing a truncating
//     accumulator), doubled again here: (d + 1) 2^-20 X B for 2 acc;
//   * products below FP32's normal range: d 1e-36 absolute.
// L2: ||bq - by||^2 = X^2 + ||by||^2 - 2 bq.by >= X^2 + K - eps, and by the
//     triangle inequality ||q - y|| >= sqrt(X^2 + K - eps) - rq - rmax = s;
//     the reference sum of d non-negative FP32 squares is at least
//     s^2 (1 - (d + 16) 2^-23).
// IP: q.y = bq.by + (q - bq).y + bq.(y - by) <= -K + eps_acc +
//     rq (B + rmax) + X rmax, and the reference -fl(q.y) loses at most
//     (d + 16) 2^-23 (X + rq)(B + rmax).
// Every margin is widened by 1 %; the caller compares strictly, so a row at
// exactly the bound cannot tie its way in.
//
// The bound arithmetic itself is FP32 with directed rounding: every
// quantity that enters as an upper bound is computed rounding up
// (__f*_ru), every lower bound rounding down (__f*_rd), so the computed
// bound is never above the exact one. Inputs outside cert_inputs_ok's range
// (where FP32 products could overflow or lose the bound) take the exact
// path instead.
#pragma once

#include <cuda_bf16.h>

namespace mv {

// Upper and lower bounds on ||bq||^2 and an upper bound on ||q - bq||^2 for
// one row (bq = the row rounded to BF16), one warp; every lane gets them.
struct CertNorms {
  float xs_lo, xs_hi, rs_hi;
};

__device__ __forceinline__ CertNorms cert_norms(const float* x, int d) {
  const int lane = threadIdx.x & 31;
  float lo = 0.0f, hi = 0.0f, rs = 0.0f;
  for (int j = lane; j < d; j += 32) {
    const float v = x[j];
    const float b = __bfloat162float(__float2bfloat16_rn(v));
    const float r = __fsub_rn(v, b);  // exact: b is v rounded to 8 significant bits
    lo = __fadd_rd(lo, __fmul_rd(b, b));
    hi = __fadd_ru(hi, __fmul_ru(b, b));
    rs = __fadd_ru(rs, __fmul_ru(r, r));
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = __fadd_rd(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = __fadd_ru(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    rs = __fadd_ru(rs, __shfl_xor_sync(0xffffffffu, rs, o));
  }
  return {lo, hi, rs};
}

// Ranges where every FP32 product of the bounds stays finite; rows outside
// them (and NaN) take the exact scan.
__device__ __forceinline__ bool cert_inputs_ok(const CertNorms& n, float B2, float rmax) {
  return B2 >= 1e-30f && B2 <= 1e30f && n.xs_lo >= 1e-30f && n.xs_hi <= 1e30f &&
         n.rs_hi <= 1e30f && rmax <= 1e15f;
}

__device__ __forceinline__ float cert_lower_l2(const CertNorms& n, float B2, float rmax, float K,
                                               int d) {
  const float B = __fsqrt_ru(B2), X = __fsqrt_ru(n.xs_hi), rq = __fsqrt_ru(n.rs_hi);
  const float c1 = __fmul_ru((float)(d + 1), 0x1p-23f), c2 = __fmul_ru((float)(d + 1), 0x1p-20f);
  const float eps = __fadd_ru(__fmul_ru(__fadd_ru(__fmul_ru(c1, B2), __fmul_ru(c2, __fmul_ru(X, B))),
                                        1.01f),
                              __fmul_ru((float)d, 1e-36f));
  const float sb = __fsub_rd(__fadd_rd(n.xs_lo, K), eps);
  const float s = __fsub_rd(__fsub_rd(sb > 0.0f ? __fsqrt_rd(sb) : 0.0f,
                                      __fmul_ru(__fadd_ru(rq, rmax), 1.01f)),
                            1e-30f);
  if (!(s > 0.0f)) return -1.0f;
  const float f = __fsub_rd(1.0f, __fmul_ru((float)(d + 16), 0x1p-23f));
  return __fmul_rd(__fmul_rd(s, s), f);
}

__device__ __forceinline__ float cert_lower_ip(const CertNorms& n, float B2, float rmax, float K,
                                               int d) {
  const float B = __fsqrt_ru(B2), X = __fsqrt_ru(n.xs_hi), rq = __fsqrt_ru(n.rs_hi);
  const float Br = __fadd_ru(B, rmax);
  const float c2 = __fmul_ru((float)(d + 1), 0x1p-20f), c3 = __fmul_ru((float)(d + 16), 0x1p-23f);
  float m = __fmul_ru(c2, __fmul_ru(X, B));
  m = __fadd_ru(m, __fmul_ru(rq, Br));
  m = __fadd_ru(m, __fmul_ru(X, rmax));
  m = __fadd_ru(m, __fmul_ru(c3, __fmul_ru(__fadd_ru(X, rq), Br)));
  return __fsub_rd(__fsub_rd(K, __fmul_ru(m, 1.01f)), __fmul_ru((float)d, 1e-36f));
}

}  // namespace mv
