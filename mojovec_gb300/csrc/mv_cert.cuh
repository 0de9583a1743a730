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
#pragma once

namespace mv {

__device__ __forceinline__ double cert_lower_l2(double X, double rq, double B2, double rmax,
                                                double K, int d) {
  const double B = sqrt(B2);
  const double eps = ((d + 1) * 0x1p-23 * B2 + (d + 1) * 0x1p-20 * X * B) * 1.01 + d * 1e-36;
  const double sb = X * X + K - eps;
  const double s = (sb > 0.0 ? sqrt(sb) : 0.0) - (rq + rmax) * 1.01 - 1e-30;
  return s > 0.0 ? s * s * (1.0 - (d + 16) * 0x1p-23) : -1.0;
}

__device__ __forceinline__ double cert_lower_ip(double X, double rq, double B2, double rmax,
                                                double K, int d) {
  const double B = sqrt(B2);
  const double m = (d + 1) * 0x1p-20 * X * B + rq * (B + rmax) + X * rmax +
                   (d + 16) * 0x1p-23 * (X + rq) * (B + rmax);
  return K - m * 1.01 - d * 1e-36;
}

}  // namespace mv
