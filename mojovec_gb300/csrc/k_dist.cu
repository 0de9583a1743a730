// Exact FP32 distance tiles in the reference's operation order.
//
// Each CTA stages a 64-row tile of X and of Y into shared memory,
// transposed (element-major) and XOR-swizzled, and every thread computes a
// 4 x 4 block of (x, y) pairs. For l2_distance_simd[8] /
// inner_product_simd[8] (utils/distances.mojo:43-228) the 32 accumulator
// lanes of the reference (4 accumulators x 8 lanes) are visited lane by
// lane: SIMD lane w of accumulator a owns elements j = 32t + 8a + w, so the
// thread forms L_w = ((acc0 + acc1) + acc2) + acc3 for each w, continues it
// through the 8-wide steps, and combines the eight lanes in reduce_add's
// halving order ((L0+L4)+(L2+L6)) + ((L1+L5)+(L3+L7)) before the 4-wide and
// scalar tails. Every operation is an explicit round-to-nearest intrinsic,
// so the result carries the reference's FP32 bits.
//
// Used by the IVF coarse quantizer (index/index_flat.mojo:260-325 with
// k = nprobe), the Flat scan, the k-means assign step
// (clustering/kmeans.mojo:114-161) and the IVF add assignment
// (index/index_ivf_pq.mojo:172).
#include "mv_exact.cuh"
#include "mv_internal.h"
#include "mv_kernels.h"

namespace mv {
namespace {

constexpr int TB = 64;   // rows per tile side
constexpr int NT = 256;  // threads per CTA (16 x 16, 4 x 4 pairs each)

__device__ __forceinline__ int swz(int j, int r) { return j * TB + (r ^ (((j >> 2) & 7) << 2)); }

__device__ __forceinline__ void stage_t(float* S, const float* A, int64_t nrows, int64_t lda,
                                        int64_t row0, int d) {
  const int total = TB * d;
  for (int e = threadIdx.x; e < total; e += NT) {
    int r = e / d;
    int j = e - r * d;
    int64_t gr = row0 + r;
    S[swz(j, r)] = (gr < nrows) ? A[gr * lda + j] : 0.0f;
  }
}

__device__ __forceinline__ void ld4(const float* S, int j, int r, float v[4]) {
  float4 t = *reinterpret_cast<const float4*>(&S[swz(j, r)]);
  v[0] = t.x;
  v[1] = t.y;
  v[2] = t.z;
  v[3] = t.w;
}

// One reference SIMD lane value for 16 pairs: L_w after the 4-accumulator
// blocks and the 8-wide steps.
template <bool IP>
__device__ __forceinline__ void lane_value(const float* Xs, const float* Ys, int T, int i0, int R8,
                                           int w, int rx, int cy, float* L) {
#pragma unroll
  for (int p = 0; p < 16; ++p) L[p] = 0.0f;
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    float acc[16];
#pragma unroll
    for (int p = 0; p < 16; ++p) acc[p] = 0.0f;
    for (int t = 0; t < T; ++t) {
      const int j = (t << 5) + (s << 3) + w;
      float xv[4], yv[4];
      ld4(Xs, j, rx, xv);
      ld4(Ys, j, cy, yv);
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          if (IP) {
            acc[a * 4 + b] = ffma(xv[a], yv[b], acc[a * 4 + b]);
          } else {
            float df = fsub(xv[a], yv[b]);
            acc[a * 4 + b] = ffma(df, df, acc[a * 4 + b]);
          }
        }
    }
#pragma unroll
    for (int p = 0; p < 16; ++p) L[p] = (s == 0) ? acc[p] : fadd(L[p], acc[p]);
  }
  for (int u = 0; u < R8; ++u) {
    const int j = i0 + (u << 3) + w;
    float xv[4], yv[4];
    ld4(Xs, j, rx, xv);
    ld4(Ys, j, cy, yv);
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        if (IP) {
          L[a * 4 + b] = ffma(xv[a], yv[b], L[a * 4 + b]);
        } else {
          float df = fsub(xv[a], yv[b]);
          L[a * 4 + b] = ffma(df, df, L[a * 4 + b]);
        }
      }
  }
}

template <int KIND>
__device__ __forceinline__ void tile_pairs(const float* Xs, const float* Ys, int d, int rx, int cy,
                                           float res[16]) {
  constexpr bool IP = (KIND == KIND_IP_SIMD8);
  if (KIND == KIND_L2_SHORT4 && d == 4) {  // distances.mojo:15-17
    float xv[4][4], yv[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      ld4(Xs, j, rx, xv[j]);
      ld4(Ys, j, cy, yv[j]);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        float r[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          float df = fsub(xv[j][a], yv[j][b]);
          r[j] = fmul(df, df);
        }
        res[a * 4 + b] = tree_sum<4>(r);
      }
    return;
  }
  if (KIND == KIND_L2_SHORT4 || d < 8) {  // scalar paths (:19-23, :57-62, :158-162)
#pragma unroll
    for (int p = 0; p < 16; ++p) res[p] = 0.0f;
    for (int j = 0; j < d; ++j) {
      float xv[4], yv[4];
      ld4(Xs, j, rx, xv);
      ld4(Ys, j, cy, yv);
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          float t;
          if (IP) {
            t = fmul(xv[a], yv[b]);
          } else {
            float df = fsub(xv[a], yv[b]);
            t = fmul(df, df);
          }
          res[a * 4 + b] = fadd(res[a * 4 + b], t);
        }
    }
    return;
  }
  const int T = d >> 5;
  const int i0 = T << 5;
  const int R8 = (d - i0) >> 3;
  int i1 = i0 + (R8 << 3);
  float A[16], B[16], C[16], D[16];
  lane_value<IP>(Xs, Ys, T, i0, R8, 0, rx, cy, A);
  lane_value<IP>(Xs, Ys, T, i0, R8, 4, rx, cy, B);
#pragma unroll
  for (int p = 0; p < 16; ++p) A[p] = fadd(A[p], B[p]);  // L0 + L4
  lane_value<IP>(Xs, Ys, T, i0, R8, 2, rx, cy, B);
  lane_value<IP>(Xs, Ys, T, i0, R8, 6, rx, cy, C);
#pragma unroll
  for (int p = 0; p < 16; ++p) A[p] = fadd(A[p], fadd(B[p], C[p]));  // + (L2 + L6)
  lane_value<IP>(Xs, Ys, T, i0, R8, 1, rx, cy, B);
  lane_value<IP>(Xs, Ys, T, i0, R8, 5, rx, cy, C);
#pragma unroll
  for (int p = 0; p < 16; ++p) B[p] = fadd(B[p], C[p]);  // L1 + L5
  lane_value<IP>(Xs, Ys, T, i0, R8, 3, rx, cy, C);
  lane_value<IP>(Xs, Ys, T, i0, R8, 7, rx, cy, D);
#pragma unroll
  for (int p = 0; p < 16; ++p) res[p] = fadd(A[p], fadd(B[p], fadd(C[p], D[p])));
  if (d - i1 >= 4) {  // 4-wide tail (:128-135 / :215-221)
    float xv[4][4], yv[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      ld4(Xs, i1 + j, rx, xv[j]);
      ld4(Ys, i1 + j, cy, yv[j]);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        float r[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (IP) {
            r[j] = ffma(xv[j][a], yv[j][b], 0.0f);
          } else {
            float df = fsub(xv[j][a], yv[j][b]);
            r[j] = fmul(df, df);
          }
        }
        res[a * 4 + b] = fadd(res[a * 4 + b], tree_sum<4>(r));
      }
    i1 += 4;
  }
  for (; i1 < d; ++i1) {  // scalar remainder
    float xv[4], yv[4];
    ld4(Xs, i1, rx, xv);
    ld4(Ys, i1, cy, yv);
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        float t;
        if (IP) {
          t = fmul(xv[a], yv[b]);
        } else {
          float df = fsub(xv[a], yv[b]);
          t = fmul(df, df);
        }
        res[a * 4 + b] = fadd(res[a * 4 + b], t);
      }
  }
}

template <int KIND>
__global__ void __launch_bounds__(NT) k_exact_matrix(const float* __restrict__ X, int64_t nx,
                                                     int64_t ldx, const float* __restrict__ Y,
                                                     int64_t ny, int64_t ldy, int d,
                                                     float* __restrict__ D, int64_t ldd) {
  extern __shared__ float sm[];
  float* Xs = sm;
  float* Ys = sm + TB * d;
  const int64_t row0 = (int64_t)blockIdx.y * TB;
  const int64_t col0 = (int64_t)blockIdx.x * TB;
  stage_t(Xs, X, nx, ldx, row0, d);
  stage_t(Ys, Y, ny, ldy, col0, d);
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int rx = ty * 4, cy = tx * 4;
  float res[16];
  tile_pairs<KIND>(Xs, Ys, d, rx, cy, res);
  const float sign = (KIND == KIND_IP_SIMD8) ? -1.0f : 1.0f;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    int64_t r = row0 + rx + a;
    if (r >= nx) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      int64_t c = col0 + cy + b;
      if (c < ny) D[r * ldd + c] = sign * res[a * 4 + b];
    }
  }
}

template <int KIND, int MODE>
__global__ void __launch_bounds__(NT) k_exact_argmin(const float* __restrict__ X, int64_t nx,
                                                     int64_t ldx, const float* __restrict__ Y,
                                                     int64_t ny, int64_t ldy, int d,
                                                     int32_t* __restrict__ amin,
                                                     float* __restrict__ amin_dist, int64_t bx,
                                                     int64_t by, int64_t ba) {
  extern __shared__ float sm[];
  __shared__ float red_d[TB][17];
  __shared__ int red_i[TB][17];
  X += blockIdx.y * bx;
  Y += blockIdx.y * by;
  amin += blockIdx.y * ba;
  if (amin_dist) amin_dist += blockIdx.y * ba;
  float* Xs = sm;
  float* Ys = sm + TB * d;
  const int64_t row0 = (int64_t)blockIdx.x * TB;
  stage_t(Xs, X, nx, ldx, row0, d);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int rx = ty * 4, cy = tx * 4;
  float best[4];
  int bidx[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    best[a] = (MODE == 1) ? 1e38f : __int_as_float(0x7f800000);
    bidx[a] = -1;
  }
  const float sign = (KIND == KIND_IP_SIMD8) ? -1.0f : 1.0f;
  for (int64_t col0 = 0; col0 < ny; col0 += TB) {
    __syncthreads();
    stage_t(Ys, Y, ny, ldy, col0, d);
    __syncthreads();
    float res[16];
    tile_pairs<KIND>(Xs, Ys, d, rx, cy, res);
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      int64_t c = col0 + cy + b;
      if (c >= ny) continue;
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        float v = sign * res[a * 4 + b];
        bool take = (MODE == 1) ? (v < best[a]) : (bidx[a] < 0 || v < best[a]);
        if (take) {
          best[a] = v;
          bidx[a] = (int)c;
        }
      }
    }
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    red_d[rx + a][tx] = best[a];
    red_i[rx + a][tx] = bidx[a];
  }
  __syncthreads();
  if (threadIdx.x < TB) {
    int r = threadIdx.x;
    float bd = 0.0f;
    int bi = -1;
    for (int t = 0; t < 16; ++t) {
      int ci = red_i[r][t];
      float cd = red_d[r][t];
      if (ci < 0) continue;
      if (bi < 0 || cd < bd || (cd == bd && ci < bi)) {
        bd = cd;
        bi = ci;
      }
    }
    int64_t gr = row0 + r;
    if (gr < nx) {
      amin[gr] = (MODE == 1) ? (bi < 0 ? 0 : bi) : bi;  // kmeans.mojo:156 max(best, 0)
      if (amin_dist) amin_dist[gr] = bd;
    }
  }
}

size_t tile_smem(int d) { return (size_t)2 * TB * d * sizeof(float); }

// Pairwise form for dimensions whose 64-row tiles do not fit shared memory:
// warp w of a CTA stages one X row, lane t computes its distance to Y row
// (blockIdx.x * 32 + t) with the same per-thread exact-order function, so
// the bits equal the tile kernel's.
template <int KIND>
__global__ void __launch_bounds__(256)
    k_exact_pairs(const float* __restrict__ X, int64_t nx, int64_t ldx, const float* __restrict__ Y,
                  int64_t ny, int64_t ldy, int d, float* __restrict__ D, int64_t ldd) {
  extern __shared__ float xs[];  // 8 rows x d
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t r = (int64_t)blockIdx.y * 8 + warp;
  const int64_t c = (int64_t)blockIdx.x * 32 + lane;
  float* xr = xs + (size_t)warp * d;
  if (r < nx)
    for (int j = lane; j < d; j += 32) xr[j] = X[r * ldx + j];
  __syncwarp();
  if (r >= nx || c >= ny) return;
  const float* yr = Y + c * ldy;
  float v;
  if (KIND == KIND_IP_SIMD8) v = -ip_simd<8>(xr, yr, d);
  else if (KIND == KIND_L2_SHORT4) v = l2_short4(xr, yr, d);
  else v = l2_simd<8>(xr, yr, d);
  D[r * ldd + c] = v;
}



template <typename K>
void set_smem(K kernel, size_t bytes) {
  smem_limit(kernel, bytes);
}

}  // namespace

void launch_exact_matrix(int kind, const float* X, int64_t nx, int64_t ldx, const float* Y,
                         int64_t ny, int64_t ldy, int d, float* D, int64_t ldd, cudaStream_t s) {
  if (nx == 0 || ny == 0) return;
  size_t smem = tile_smem(d);
  if (smem > 200 * 1024) {  // large d: the pairwise form
    const size_t ps = (size_t)8 * d * sizeof(float);
    MV_REQUIRE(ps <= 200 * 1024, MV_ERR_UNSUPPORTED, "exact distances: dimension too large");
    MV_REQUIRE((nx + 7) / 8 <= 65535, MV_ERR_UNSUPPORTED, "too many query rows in one call");
    dim3 pg((unsigned)((ny + 31) / 32), (unsigned)((nx + 7) / 8));
    auto go = [&](auto kernel) {
      set_smem(kernel, ps);
      kernel<<<pg, 256, ps, s>>>(X, nx, ldx, Y, ny, ldy, d, D, ldd);
    };
    if (kind == KIND_IP_SIMD8) go(k_exact_pairs<KIND_IP_SIMD8>);
    else if (kind == KIND_L2_SHORT4) go(k_exact_pairs<KIND_L2_SHORT4>);
    else go(k_exact_pairs<KIND_L2_SIMD8>);
    count_launch();
    MV_CHECK_CUDA(cudaGetLastError());
    return;
  }
  MV_REQUIRE((nx + TB - 1) / TB <= 65535, MV_ERR_UNSUPPORTED, "too many query rows in one call");
  dim3 grid((unsigned)((ny + TB - 1) / TB), (unsigned)((nx + TB - 1) / TB));
  switch (kind) {
    case KIND_L2_SIMD8:
      set_smem(k_exact_matrix<KIND_L2_SIMD8>, smem);
      k_exact_matrix<KIND_L2_SIMD8><<<grid, NT, smem, s>>>(X, nx, ldx, Y, ny, ldy, d, D, ldd);
      break;
    case KIND_IP_SIMD8:
      set_smem(k_exact_matrix<KIND_IP_SIMD8>, smem);
      k_exact_matrix<KIND_IP_SIMD8><<<grid, NT, smem, s>>>(X, nx, ldx, Y, ny, ldy, d, D, ldd);
      break;
    default:
      set_smem(k_exact_matrix<KIND_L2_SHORT4>, smem);
      k_exact_matrix<KIND_L2_SHORT4><<<grid, NT, smem, s>>>(X, nx, ldx, Y, ny, ldy, d, D, ldd);
  }
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

void launch_exact_argmin(int kind, int mode, const float* X, int64_t nx, int64_t ldx,
                         const float* Y, int64_t ny, int64_t ldy, int d, int32_t* amin,
                         float* amin_dist, int batch, int64_t bx, int64_t by, int64_t ba,
                         cudaStream_t s) {
  if (nx == 0 || batch == 0) return;
  size_t smem = tile_smem(d);
  MV_REQUIRE(smem <= 200 * 1024, MV_ERR_UNSUPPORTED, "exact distance tile: dimension too large");
  MV_REQUIRE(batch <= 65535, MV_ERR_UNSUPPORTED, "argmin batch too large");
  dim3 grid((unsigned)((nx + TB - 1) / TB), (unsigned)batch);
#define MV_ARGMIN_CASE(K, Mo)                                                                 \
  do {                                                                                        \
    set_smem(k_exact_argmin<K, Mo>, smem);                                                    \
    k_exact_argmin<K, Mo><<<grid, NT, smem, s>>>(X, nx, ldx, Y, ny, ldy, d, amin, amin_dist, \
                                                 bx, by, ba);                                 \
  } while (0)
  if (mode == 1) {
    if (kind == KIND_L2_SIMD8) MV_ARGMIN_CASE(KIND_L2_SIMD8, 1);
    else if (kind == KIND_IP_SIMD8) MV_ARGMIN_CASE(KIND_IP_SIMD8, 1);
    else MV_ARGMIN_CASE(KIND_L2_SHORT4, 1);
  } else {
    if (kind == KIND_L2_SIMD8) MV_ARGMIN_CASE(KIND_L2_SIMD8, 2);
    else if (kind == KIND_IP_SIMD8) MV_ARGMIN_CASE(KIND_IP_SIMD8, 2);
    else MV_ARGMIN_CASE(KIND_L2_SHORT4, 2);
  }
#undef MV_ARGMIN_CASE
  count_launch();
  MV_CHECK_CUDA(cudaGetLastError());
}

}  // namespace mv
