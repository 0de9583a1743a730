// Host interface of the BF16 tensor-core distance GEMM (k_umma.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace mv {

enum UmmaEpilogue : int {
  EPI_MATRIX = 0,  // write the distance matrix
  EPI_ARGMIN = 1,  // per-row min (distance, column) key via atomicMin
};

struct UmmaArgs {
  int64_t nrows, ncols;
  int nkb;           // 64-element k-blocks
  int metric;        // MV_METRIC_L2 / MV_METRIC_IP
  const float* rnorm;  // ||x||^2 per row (may be null: row-constant term dropped)
  const float* cnorm;  // ||y||^2 per column (L2)
  float* out;
  int64_t ldo;
  uint64_t* keys;    // EPI_ARGMIN output, one per row
  int* err;          // set to 1 when a bounded wait gave up
  long long wait_limit = 4000000000ll;  // cycles per pipeline wait (the context's setting)
};

struct UmmaTopkArgs {
  int64_t nrows, ncols;
  int nkb, metric;
  const float* rnorm;  // may be null
  const float* cnorm;
  int nc, ncp;         // keys kept per row, padded output stride (power of two)
  int nseg, tps;       // column segments (grid.x) and column tiles per segment
  int pend;            // pending keys per row (multiple of 8, >= 32)
  const uint8_t* filter;  // filter[col] > 0 excludes the column (may be null)
  uint64_t* gthr;      // per-row threshold shared by the segments (may be null)
  uint64_t* out;       // nrows x nseg x ncp keys (distance, column)
  int* err;
  const float* rscale = nullptr;  // E4M3 operands: per-row scale of X
  const float* cscale = nullptr;  // E4M3 operands: per-column scale of Y
  long long wait_limit = 4000000000ll;  // cycles per pipeline wait (the context's setting)
};

struct CoarseTopkArgs {
  int64_t nrows, ncols;
  int nkb;
  const float* cnorm;  // ||y||^2 per column (L2)
  int nc;              // keys kept per row
  int nseg, tps;       // column segments (grid.x) and 128-column tiles per segment
  int cap;             // list slots per row and segment (> nc)
  uint64_t* lists;     // nrows x nseg x cap keys (distance, column)
  int* counts;         // nrows x nseg
  uint32_t* gthr;      // per-row threshold shared by the segments (may be null)
  int* err;
  long long wait_limit = 4000000000ll;  // cycles per pipeline wait (the context's setting)
};

// Rows are padded to this many BF16 elements (a multiple of 64).
int umma_kpad(int d);
// E4M3 rows are padded to this many bytes (a multiple of 128).
int umma_kpad8(int d);
// FP32 rows -> E4M3 rows scaled to the format's range (x = scale * x8,
// scale = max|x| / 448 per row, round to nearest, saturating), zero padded
// to umma_kpad8(d); norms of the dequantized rows (may be null).
void launch_to_e4m3(const float* x, int64_t n, int d, uint8_t* out, float* scales, float* norms,
                    cudaStream_t s);
// FP32 rows -> zero-padded BF16 rows (kpad wide) and FP32 norms of the
// rounded rows (norms may be null).
void launch_to_bf16(const float* x, int64_t n, int d, __nv_bfloat16* out, float* norms,
                    cudaStream_t s);
// Distances between BF16 rows X (nx) and Y (ny) on the tensor cores.
void launch_umma_dist(int epi, const __nv_bfloat16* X, int64_t nx, const __nv_bfloat16* Y,
                      int64_t ny, int d, int metric, const float* xnorm, const float* ynorm,
                      float* out, int64_t ldo, uint64_t* keys, int* err, int num_sms,
                      cudaStream_t s);
// Most keys the fused top-k GEMM keeps per row and column segment.
constexpr int UMMA_TOPK_MAX = 64;
// Longest padded row (elements) the fused top-k GEMM takes; above 256 the X
// block streams through shared memory with the Y tiles.
constexpr int UMMA_TOPK_MAX_K = 2048;
// Epilogue groups of the fused top-k GEMM for (d, nc): each CTA writes one
// output segment per group, so a launch with nseg column segments leaves
// nseg * groups segments per row.
int umma_topk_groups(int d, int nc, bool e4m3 = false);
// Column segments for the fused top-k GEMM: enough CTAs to fill the SMs
// in whole waves.
int umma_topk_nseg(int64_t nrows, int64_t ncols, int d, int nc, int num_sms, bool e4m3 = false);
// Per-row nc smallest (distance, column) keys of the BF16 distances, per
// output segment: out[(row * S + s) * next_pow2(nc) + j] with
// S = nseg * umma_topk_groups(d, nc), unsorted, KEY_NONE padded. The key
// distance leaves out the row's own ||x||^2.
// gthr (nx keys, may be null) lets the segments share the row threshold;
// only valid when the caller needs no more than nc keys per row.
void launch_umma_topk(const __nv_bfloat16* X, int64_t nx, const __nv_bfloat16* Y, int64_t ny,
                      int d, int metric, const float* xnorm, const float* ynorm, int nc, int nseg,
                      const uint8_t* filter, uint64_t* gthr, uint64_t* out, int* err,
                      cudaStream_t s);
// The same with E4M3 operands (kind::f8f6f4): X8 nx x umma_kpad8(d) with
// per-row scales xscale, Y8 with per-column scales yscale and ynorm the
// norms of the dequantized Y rows (L2). The key distance is
// ||y||^2 - 2 sx sy <x8, y8> (L2) or -sx sy <x8, y8> (IP).
void launch_umma_topk_e4m3(const uint8_t* X8, int64_t nx, const float* xscale, const uint8_t* Y8,
                           int64_t ny, const float* yscale, int d, int metric, const float* ynorm,
                           int nc, int nseg, const uint8_t* filter, uint64_t* gthr, uint64_t* out,
                           int* err, cudaStream_t s);
// Two-pass coarse top-nc GEMM (d <= 256, nc <= 32): per row and column
// segment, a list of at most coarse_topk2_cap(nc) unsorted keys
// lists[(row * nseg + seg) * cap + j], j < counts[row * nseg + seg], that
// contains the segment's nc smallest (distance, column) keys of the BF16
// distances (the keys launch_umma_topk keeps; the key distance leaves out
// the row's own ||x||^2).
int coarse_topk2_cap(int nc);
int coarse_topk2_nseg(int64_t nrows, int64_t ncols, int d, int nc, int num_sms);
// gthr: nx words of scratch (used when nseg > 1).
void launch_coarse_topk2(const __nv_bfloat16* X, int64_t nx, const __nv_bfloat16* Y, int64_t ny,
                         int d, int metric, const float* ynorm, int nc, int nseg, uint64_t* lists,
                         int* counts, uint32_t* gthr, int* err, cudaStream_t s);
// keys -> argmin columns (and distances).
void launch_keys_argmin(const uint64_t* keys, int64_t n, int32_t* out, float* dist, cudaStream_t s);

}  // namespace mv
