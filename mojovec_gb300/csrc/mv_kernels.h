// Kernel launchers shared by the C-ABI layer. Each launcher enqueues on the
// given stream and throws mv::Error on a launch failure.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace mv {

void count_launch();  // increments the owning context's launch counter

// Distance kinds used by the plain kernels.
enum DistKind : int {
  KIND_L2_SIMD8 = 0,   // l2_distance_simd[8]
  KIND_IP_SIMD8 = 1,   // -inner_product_simd[8] (IndexFlat IP distance)
  KIND_L2_SHORT4 = 2,  // l2_distance_short4 (k-means with d <= 4, PQ dsub <= 4)
};

// ---- exact distances (k_dist.cu) -----------------------------------------
// kind: 0 = l2_distance_simd[8], 1 = -inner_product_simd[8], 2 = l2_short4.
// D[i][j] = dist(X[i], Y[j]) for i < nx, j < ny.
void launch_exact_matrix(int kind, const float* X, int64_t nx, int64_t ldx, const float* Y,
                         int64_t ny, int64_t ldy, int d, float* D, int64_t ldd, cudaStream_t s);
// amin[i] = argmin_j dist(X[i], Y[j]); mode 1 = k-means (strict `<` from
// 1e38, -1 -> 0), mode 2 = IndexFlat k = 1 heap (first element always in).
// Batched over `batch` problems with element strides bx, by, ba.
void launch_exact_argmin(int kind, int mode, const float* X, int64_t nx, int64_t ldx,
                         const float* Y, int64_t ny, int64_t ldy, int d, int32_t* amin,
                         float* amin_dist, int batch, int64_t bx, int64_t by, int64_t ba,
                         cudaStream_t s);

// ---- selection (k_select.cu) ---------------------------------------------
// For each row r < rows: k smallest (D[r][c], col_base + c) keys over
// c < ncols, merged with prev[r][0..k) when prev != nullptr. filter[gid] > 0
// excludes column gid (may be nullptr).
void launch_select_rows(const float* D, int64_t rows, int64_t ldd, int64_t ncols,
                        int64_t col_base, int k, const uint64_t* prev, uint64_t* out,
                        const uint8_t* filter, cudaStream_t s);
// keys (rows x k) -> distances / labels; empty slots get fill_d / -1;
// negate flips the sign of found distances (IP un-negation).
void launch_keys_to_results(const uint64_t* keys, int64_t rows, int k, float fill_d, bool negate,
                            float* out_d, int64_t* out_l, cudaStream_t s);
// keys (rows x k) -> int32 ids (empty -> -1).
void launch_keys_to_ids(const uint64_t* keys, int64_t n, int32_t* out, cudaStream_t s);

// ---- IVF-PQ (k_ivfpq.cu) -------------------------------------------------
struct IvfpqScanArgs {
  const float* q;
  int64_t nq;
  int d, M, dsub, metric;
  const float* centroids;
  const float* pq;
  const int64_t* list_off;
  const uint32_t* ids;
  const uint8_t* codes;
  const int32_t* probes;
  int nprobe;
  const uint8_t* filter;
  int64_t filter_len;
  int k;
  float* out_d;
  int64_t* out_l;
};
void launch_ivfpq_scan_plain(const IvfpqScanArgs& a, cudaStream_t s);
// residual[i] = x[i] - centroids[assign[i]] (assign < 0 or >= nlist -> 0).
void launch_residuals(const float* x, int64_t n, int d, const float* centroids, int nlist,
                      const int32_t* assign, float* out, cudaStream_t s);
// ProductQuantizer.compute_codes on residual rows.
void launch_pq_encode(const float* x, int64_t n, int d, int M, const float* pq, uint8_t* codes,
                      cudaStream_t s);
// ProductQuantizer.compute_distance_table for nq rows: out nq x M x 256.
void launch_pq_tables(const float* x, int64_t nq, int d, int M, const float* pq, int metric,
                      float* out, cudaStream_t s);
// [n x d] -> [M x n x dsub] (subspace extraction, pq.mojo:58-62).
void launch_split_subspaces(const float* x, int64_t n, int d, int M, float* out, cudaStream_t s);

// ---- list append (k_lists.cu) -------------------------------------------
// Rebuilt-CSR positions for an append of n entries with list numbers
// assign[i] (outside [0, nlist): skipped, parked past the end): pos[0,
// old_total) for the old entries, pos[old_total, old_total + n) for the new
// ones in input order; new_off[nlist + 1]. scratch: list_append_scratch_bytes.
size_t list_append_scratch_bytes(int64_t n, int nlist);
void launch_list_append_layout(const int32_t* assign, int64_t n, int nlist, const int64_t* old_off,
                               int64_t old_total, int64_t* new_off, int64_t* pos, void* scratch,
                               cudaStream_t s);

// ---- certified exact selections (k_assign.cu) ---------------------------
// cert[0] = bound on ||bf16(y)||^2 over the n rows (from their FP32 norms of
// the BF16 rows; -1 when one is NaN or infinite), cert[1] = max over rows of
// ||y - bf16(y)||.
void launch_cert_bounds(const float* norms, const float* rows, int64_t n, int d, float* cert,
                        cudaStream_t s);
// Exact recheck of the top-k GEMM candidates (cand: n x ncand keys) with the
// reference distance (l2_simd<8> / -ip_simd<8>), best candidate to assign[],
// and rows the error bound does not settle appended to flagged[] (count in
// *nflag).
void launch_assign_certify(const float* x, int64_t n, int d, const float* cent, int nlist, int metric,
                           const uint64_t* cand, int ncand, int kc, const float* cert,
                           int32_t* assign, float* mind, int64_t* flagged, int* nflag,
                           cudaStream_t s);
// The P nearest centroids per row (ascending (distance, list)) from the
// GEMM's candidates; rows the bound does not settle go to flagged[].
void launch_topp_certify(const float* x, int64_t n, int d, const float* cent, int nlist, int metric,
                         const uint64_t* cand, int ncand, int kc, int P, const float* cert,
                         int32_t* probes, int64_t* flagged, int* nflag, cudaStream_t s);
// Flat top-k from each query's shortlist of R approximate keys: reference
// distances, the k smallest written (0.0 / -1 tail, IP un-negated), flag[q]
// = 1 when the bound (or over[q], may be null) leaves the query open.
size_t flat_certify_smem(int d, int R, int k);
void launch_flat_certify(const float* q, int64_t nq, int d, int metric, const float* rows,
                         int64_t nb, const uint64_t* skeys, int R, int k, const float* cert,
                         const int* over, float* out_d, int64_t* out_l, int* flag,
                         cudaStream_t s);
// assign[idx[i]] = sub[i] (and mind[idx[i]] = sub_d[i] when mind is not null).
void launch_scatter_assign(const int32_t* sub, const float* sub_d, const int64_t* idx, int64_t count,
                           int32_t* assign, float* mind, cudaStream_t s);

// ---- k-means (k_kmeans.cu) -----------------------------------------------
// Gathers rows: out[i] = x[idx[i]].
void launch_gather_rows(const float* x, int d, const int64_t* idx, int64_t count, float* out,
                        int batch, int64_t bx, int64_t bo, cudaStream_t s);
// Per-chunk FP32 row sums in row order (kmeans.mojo:114-161) and counts.
void launch_kmeans_accumulate(const float* x, int64_t n, int d, int k, const int32_t* assign,
                              float* local_sums, int32_t* local_counts, int batch, int64_t bx,
                              int64_t ba, int64_t bs, int64_t bc, cudaStream_t s);
// Ordered chunk reduce + reciprocal-multiply update + reseed (:170-220).
void launch_kmeans_update(const float* x, int64_t n, int d, int k, const float* local_sums,
                          const int32_t* local_counts, int64_t sample_offset, int iteration,
                          float* centroids, int batch, int64_t bx, int64_t bs, int64_t bc,
                          int64_t bcent, cudaStream_t s);
void launch_i32_to_i64(const int32_t* a, int64_t n, int64_t* out, cudaStream_t s);

// ---- SQ8 (k_sq8.cu) ------------------------------------------------------
// out2 = {min, max} over n values (initialised by the launcher).
void launch_minmax(const float* x, int64_t n, float* out2, cudaStream_t s);
// _encode_sq8_vector for rows (sq8.mojo:13-38); codes rows are dpad bytes,
// zero padded.
void launch_sq8_encode(const float* x, int64_t n, int d, int dpad, float minimum, float inv_scale,
                       bool symmetric, uint8_t* codes, uint32_t* norms, cudaStream_t s);
// Distances between query codes and base codes (sq8.mojo:62-79).
// ---- fast k-means (k_kmeans_fast.cu) ---------------------------------------
// Exact FP32 pick among ncand candidate keys per row (reference distance and
// tie rule): assign[r], mind[r].
void launch_km_recheck(const float* x, int64_t n, int d, const float* cent, int k,
                       const uint64_t* cand, int ncand, int32_t* assign, float* mind,
                       cudaStream_t s);
size_t km_sort_scratch_bytes(int64_t n, int k);
// Deterministic FP64 centroid update (stable counting sort + ordered sums).
void launch_km_update_fp64(const float* x, int64_t n, int d, int k, const int32_t* assign,
                           int64_t sample_offset, int it, float* cent, void* scratch,
                           cudaStream_t s);
// out = sum of v in FP64 in a fixed order (part256: 256 doubles of scratch).
void launch_sum_fp64(const float* v, int64_t n, double* part256, double* out, cudaStream_t s);

// IVF-Flat scan of the probed lists (k_ivfflat.cu).
void launch_ivfflat_scan(const float* q, int64_t nq, int d, int metric, const int32_t* probes,
                         int nprobe, int nlist, const int64_t* list_off, const float* rows,
                         const uint32_t* ids, int k, float* out_d, int64_t* out_l, cudaStream_t s);
// List-major form of the same scan (k <= 32): (query, probe) pairs grouped
// by list, each list read once per 4 of its queries; same results.
// scratch: ivfflat_lm_scratch_bytes() bytes of device memory.
size_t ivfflat_lm_scratch_bytes(int64_t nq, int nprobe, int nlist, int k);
bool ivfflat_lm_supported(int64_t nq, int d, int nprobe, int k);
void launch_ivfflat_scan_lm(const float* q, int64_t nq, int d, int metric, const int32_t* probes,
                            int nprobe, int nlist, const int64_t* list_off, const float* rows,
                            const uint32_t* ids, int k, float* out_d, int64_t* out_l, void* scratch,
                            cudaStream_t s);

// SQ8 codes as BF16 rows (kp wide) and FP32 norms, for the tensor-core scan.
void launch_sq8_codes_to_bf16(const uint8_t* codes, int64_t n, int d, int dpad, int kp,
                              bool symmetric, const uint32_t* norms, __nv_bfloat16* out,
                              float* fnorms, cudaStream_t s);
void launch_sq8_matrix(const uint8_t* qc, const uint32_t* qn, int64_t nq, const uint8_t* bc,
                       const uint32_t* bn, int64_t nb, int dpad, bool ip, float scale_sq,
                       float* D, int64_t ldd, cudaStream_t s);
// Exact FP32 rerank of candidate ids (cand rows x ncand, -1 = none) with
// l2_distance_simd[64] / -inner_product_simd[64]; keys out rows x k.
void launch_rerank_simd64(const float* q, int64_t nq, int d, const float* base, int64_t nb, int metric,
                          const int64_t* cand, int ncand, int k, uint64_t* out_keys,
                          cudaStream_t s);

// ---- misc ----------------------------------------------------------------
// _normalize_vectors in FP64; bad[0] set to 1 (non-finite) or 2 (zero row).
void launch_normalize(const float* x, int64_t n, int d, float* out, int32_t* bad, cudaStream_t s);

}  // namespace mv
