// Host interface of the fast-form IVF-PQ kernels (k_ivfpq_fast.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cuda_runtime.h>

#include <cstdint>

namespace mv {

struct FastScanArgs {
  const float* q;
  int64_t nq;
  int d, M, metric;
  const float* pq;
  // FP16 codebook scaled by a power of two (pq16 = pq / pq16_inv; dsub 4 or
  // 8), read instead of pq when set: the table values differ from FP32 ones
  // by the FP16 rounding of the codewords.
  const __half* pq16 = nullptr;
  float pq16_inv = 1.0f;
  // Per subspace, an upper bound on the largest codeword norm; when set the
  // scan uses the bank-rotated integer tables (M a multiple of 4, M >= 8).
  const float* pq_cn = nullptr;
  const int64_t* list_off;
  const uint8_t* codes;
  const float* vterm;     // per CSR entry, null for IP
  const int32_t* probes;  // nq x nprobe, ascending coarse distance
  const float* term;      // nq x nprobe coarse distances (exact FP32)
  int nprobe;
  int R;                  // shortlist length
  int sorted;             // 1: shortlist sorted ascending (it is the answer)
  uint64_t* out_keys;     // nq x R (distance, CSR position)
  int nlist;              // bounds of the data-dependent indices
  int64_t ntotal;
  int* err;               // set to a site code if an index is out of range
  const int32_t* nprobe_q = nullptr;  // per-query nprobe (<= nprobe), may be null
  const int32_t* order = nullptr;     // scan order of the queries, may be null
  int* counter = nullptr;             // persistent grid: next position in `order`
  // index_ivf_pq.mojo:328-334: an entry whose id is below filter_len and has
  // filter[id] != 0 is skipped (ids: the id of each CSR entry)
  const uint8_t* filter = nullptr;
  int64_t filter_len = 0;
  const uint32_t* ids = nullptr;
  int cap, Rp;            // set by the launcher
  int rot = 0;            // set by the launcher: rotated-table pass width (0: none)
  int stage_entries = 0;  // staged scan: candidates per staged round (0: automatic)
};

struct RerankArgs {
  const float* q;
  int64_t nq;
  int d, metric;
  const float* raw;       // FP32 rows in CSR order
  const uint32_t* ids;    // id per CSR entry (null: the position is the id)
  const uint64_t* cand;   // nq x R shortlist keys
  int R, k;
  float* out_d;
  int64_t* out_l;
  int64_t ntotal;         // CSR entries (bound of the shortlist positions)
  int* err;
  float fill_d = 1e38f;   // distance of an unfilled slot (label -1)
  const int32_t* k_q = nullptr;  // per-query k (<= k; the row keeps k slots), may be null
  int kp;                 // set by the launcher
  // Certified prescreen (k <= 32; all null: every candidate is computed in
  // FP32): BF16 copies of the rows, per row an upper bound on
  // ||y - bf16(y)|| and (IP) on ||bf16(y)||.
  const __nv_bfloat16* raw16 = nullptr;
  const float* rad = nullptr;
  const float* n16 = nullptr;
};

// BF16 copies of FP32 rows (CSR order) for the certified rerank prescreen,
// with per row upper bounds on ||y - bf16(y)|| and ||bf16(y)||.
void launch_rerank_rows(const float* raw, int64_t n, int d, __nv_bfloat16* raw16, float* rad,
                        float* n16, cudaStream_t s);

// Two-pass coarse GEMM lists (launch_coarse_topk2) -> the nprobe nearest
// lists, as launch_coarse_rows (one warp per query; nseg * cap <= 256).
// The same lists -> each row's nc (<= 32) smallest keys, sorted, padded with
// KEY_NONE to next_pow2(nc) per row.
void launch_lists_smallest(const uint64_t* lists, const int* counts, int nseg, int cap, int64_t nq,
                           int nc, uint64_t* out, cudaStream_t s);
void launch_coarse_lists(const uint64_t* lists, const int* counts, int nseg, int cap, int64_t nq,
                         int nlist, const float* q, int d, const float* cent, int metric, int nc,
                         int nprobe, int32_t* probes, float* term, int* err, cudaStream_t s);
void launch_vec_terms(const int64_t* off, int nlist, const uint8_t* codes, const float* pq,
                      const float* cent, int d, int M, float* out, cudaStream_t s);
// Top-nc of the approximate coarse distances, exact FP32 recheck, top-nprobe.
void launch_coarse_fast(const float* approx, int64_t nq, int nlist, const float* q, int d,
                        const float* cent, int metric, int nc, int nprobe, int32_t* probes,
                        float* term, int* err, cudaStream_t s);
// Same with one warp per query and a lane-minimum threshold (nc <= 64).
void launch_coarse_rows(const float* approx, int64_t nq, int nlist, const float* q, int d,
                        const float* cent, int metric, int nc, int nprobe, int32_t* probes,
                        float* term, int* err, cudaStream_t s);
// Same from per-row candidate keys (ncand per row, KEY_NONE padded).
void launch_coarse_from_keys(const uint64_t* cand, int64_t nq, int ncand, const float* q, int d,
                             const float* cent, int nlist, int metric, int nc, int nprobe,
                             int32_t* probes, float* term, int* err, cudaStream_t s);
size_t fast_scan_smem(const FastScanArgs& a);
// The staged scan (k_ivfpq_scan.cu); returns false, launching nothing, when
// its shared memory would not fit (the caller runs the unstaged kernel).
bool launch_ivfpq_scan_staged(FastScanArgs a, cudaStream_t s, int nt, int persistent_ctas, int E);
// lut: 0 or 2 = FP32 tables read with codes from global memory, 1 = FP16
// tables with a per-query power-of-two scale (FP32 sums), 3 = bank-rotated
// fixed-point tables where M allows (else FP32), 4 = FP32 tables with codes
// and terms staged in shared memory by bulk copies (the unstaged kernel when
// that does not fit).
void launch_ivfpq_scan_fast(FastScanArgs a, cudaStream_t s, int nt = 256, int persistent_ctas = 0,
                            int lut = 0);
// List-major ADC on the tensor cores (k_ivfpq_tc.cu): FP16 queries times
// FP16 reconstructions of the list rows, one decode per list row and batch;
// writes the R smallest (distance, position) keys per query like the scan
// above (a.q, nq, d, M, metric, pq16, pq16_inv, list_off, codes, vterm,
// probes, term, nprobe, nprobe_q, R, sorted, out_keys, nlist, err, filter).
// Shapes: FP16 codebook, M a multiple of 8, d / M = 4 or 8, d <= 128.
bool ivfpq_tc_supported(int d, int M, bool has_pq16);
// Queries per work item (64 or 128) for a batch shape.
int ivfpq_tc_qc(int64_t nq, int nprobe, int nlist);
// smax: an upper bound on any query's candidate count (the nprobe longest
// lists); the scratch holds nq distance rows of smax words, the query
// images of the work items and one flag per CSR row (ntotal).
size_t ivfpq_tc_scratch_bytes(int64_t nq, int nprobe, int nlist, int d, int64_t smax, int qc,
                              int64_t ntotal);
void launch_ivfpq_scan_tc(const FastScanArgs& a, int64_t smax, int qc, void* scratch, int num_sms,
                          long long wait_limit, cudaStream_t s);
// Flat fast form: merge nseg x ncp per-segment keys (kseg kept per segment)
// into the R-key shortlist per query. With out_keys the shortlist is
// written (unsorted) for the rerank; otherwise the k smallest become the
// results (L2 adds qnorm back). overflow[q] = 1 when a segment may have
// dropped a shortlist key (only possible when kseg < R); may be null.
// SQ8 tensor-core scan: per-segment (-e, row) keys -> the R smallest
// canonical (SQ8 distance, row) keys per query (unsorted, KEY_NONE padded);
// flag[q] = 1 when a dropped row could tie into the shortlist.
void launch_sq8_merge(const uint64_t* cand, int64_t nq, int nseg, int ncp, int kseg, int R,
                      const uint32_t* qnorm, bool ip, float scale_sq, uint64_t* out_keys, int* flag,
                      cudaStream_t s);
void launch_flat_merge(const uint64_t* cand, int64_t nq, int nseg, int ncp, int kseg, int R,
                       uint64_t* out_keys, int k, const float* qnorm, int metric, float fill_d,
                       float* out_d, int64_t* out_l, int* overflow, cudaStream_t s);
void launch_rerank_fast(RerankArgs a, cudaStream_t s);
void launch_short_to_results(const uint64_t* keys, int64_t nq, int R, int k, const uint32_t* ids,
                             int metric, float* out_d, int64_t* out_l, cudaStream_t s,
                             const int32_t* k_q = nullptr);

}  // namespace mv
